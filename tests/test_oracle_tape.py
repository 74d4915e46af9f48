"""The oracle port's decision tape (CPU): recording changes no bit of a run,
replaying the record on the same inputs gives the same run, and on perturbed
inputs the replayed run follows the base run's branches (it differs from a
free run exactly where a decision would have switched).  The tape makes the
perturbed forward maps of the adjoint's finite-difference check smooth."""
import numpy as np

from oracle import Problem


def _case(n=(14, 12, 10), seed=3):
    pb = Problem(nx=n[0], ny=n[1], nz=n[2], dim=3, s_l=0.2, dt=2e-3, enable_reinit=True, reinit_interval=2,
                 reinit_iterations=2)
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(*[(np.arange(q + 6) - 3) / q for q in n[::-1]], indexing="ij")
    G = np.sqrt((x - 0.5) ** 2 + (y - 0.45) ** 2 + (z - 0.5) ** 2) - 0.3 + 0.01 * rng.standard_normal(pb.shape)
    vel = [rng.standard_normal(pb.shape) for _ in range(3)]
    sl = 0.15 + 0.05 * rng.random(pb.shape)
    return pb, np.ascontiguousarray(G), vel, sl


def test_tape_record_and_replay(port):
    pb, G, vel, sl = _case()
    steps = 5
    cells = pb.nx * pb.ny * pb.nz
    stage = np.zeros((3 * steps, cells), np.uint8)
    pseudo = np.zeros((2 * 2, cells), np.uint8)
    flags = np.zeros((2, cells), np.uint8)
    free = port.run(pb, steps, G, *vel, sl=sl)
    port.tape("record", stage, pseudo, flags)
    rec = port.run(pb, steps, G, *vel, sl=sl)
    assert port.tape_counts() == (3 * steps, 4, 2, 0)
    port.tape("replay", stage, pseudo, flags)
    rep = port.run(pb, steps, G, *vel, sl=sl)
    port.tape("off")
    assert np.array_equal(rec, free) and np.array_equal(rep, free)
    assert stage.any() and (stage != 7).any() and flags.any()  # both upwind directions and crossings occur
    # a perturbed replay stays on the base branches: close to the free perturbed
    # run, equal where no decision switched, and a smooth function of the step
    d = np.random.default_rng(9).standard_normal(sl.shape)
    outs = []
    for h in (1e-6, 2e-6):
        port.tape("replay", stage, pseudo, flags)
        outs.append(port.run(pb, steps, G, *vel, sl=sl + h * d))
        port.tape("off")
    # second difference: O(h^2) plus rounding on a smooth map; a switched
    # branch would leave a jump of the order of the first difference
    first = np.abs(outs[0] - free).max()
    lin = outs[1] - free - 2 * (outs[0] - free)
    assert first > 0 and np.abs(lin).max() < 1e-3 * first
