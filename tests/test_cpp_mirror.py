"""The C++ mirror of the reference's function surface (include/lsgb_levelset.hpp).

CPU: the header compiles against a caller-side SimParams with the reference's
member names.  GPU: a C++ driver written like the reference's main loop runs
through it and reproduces the reference's golden output bit for bit."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "mirror_check.cpp")
SAMPLE_SRC = os.path.join(ROOT, "tests", "cpp", "sample_check.cpp")
INC = [os.path.join(ROOT, "include"), "/usr/local/cuda/include"]


def test_mirror_header_compiles():
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    for src in (SRC, SAMPLE_SRC):
        cmd = [gxx, "-std=c++14", "-fsyntax-only", *sum((["-I", i] for i in INC), []), src]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_mirror_reproduces_reference_golden(cuda, lsgb_mod, tmp_path):
    z = np.load(os.path.join(ROOT, "tests", "golden", "golden_3d_small.npz"))
    files = []
    for name in ("G", "u", "v", "w"):
        path = tmp_path / f"{name}.bin"
        np.ascontiguousarray(z[name]).tofile(path)
        files.append(str(path))
    exe = tmp_path / "mirror_check"
    libdir = os.path.dirname(lsgb_mod.LIB_PATH)
    cmd = ["g++", "-std=c++14", "-O2", *sum((["-I", i] for i in INC), []), SRC, "-o", str(exe),
           "-L", libdir, "-llsgb", f"-Wl,-rpath,{libdir}", "-L/usr/local/cuda/lib64", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = tmp_path / "out.bin"
    dump = tmp_path / "G_final.bin"
    r = subprocess.run([str(exe), *files, str(out), "12", "10", "8", repr(float(z["s_l"])),
                        repr(float(z["dt"])), "10", str(dump)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    G = np.fromfile(out, dtype=np.float64).reshape(z["run10"].shape)
    assert np.array_equal(G, z["run10"])
    vol = float(r.stdout.split()[1])
    assert vol == pytest.approx(float(z["vol_run10"]), rel=1e-12)
    with open(os.path.join(ROOT, "tests", "golden", "dump_3d_small_run10.bin"), "rb") as f:
        assert dump.read_bytes() == f.read()


@pytest.mark.gpu
def test_sample_mirror_matches_oracle(cuda, lsgb_mod, tmp_path):
    """sample/main.cpp's loop written against lsgb_sample.hpp: the interior
    dump equals the oracle port's run (which equals the reference's own
    sources) bit for bit."""
    from oracle import SampleOracle
    from lsgb import sample as smp
    nx, ny, dt, steps, freq = 40, 32, 1e-4, 17, 60
    G0 = smp.bunsen(nx, ny)
    g0 = tmp_path / "G0.bin"
    G0.tofile(g0)
    exe = tmp_path / "sample_check"
    libdir = os.path.dirname(lsgb_mod.LIB_PATH)
    cmd = ["g++", "-std=c++14", "-O2", "-ffp-contract=off", *sum((["-I", i] for i in INC), []), SAMPLE_SRC,
           "-o", str(exe), "-L", libdir, "-llsgb", f"-Wl,-rpath,{libdir}", "-L/usr/local/cuda/lib64", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), str(g0), str(out), str(nx), str(ny), repr(dt), str(steps), str(freq)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    dx, dy = smp.spacing(nx, ny)
    ref, t = SampleOracle("port").run(G0, G0, steps, dx, dy, dt, smp.SL, smp.U0, smp.V0, smp.EPS_U, smp.EPS_V, freq)
    dump = np.fromfile(out, dtype=np.float64).reshape(ny, nx)
    assert np.array_equal(dump, ref[3:-3, 3:-3])
    assert float(r.stdout.split()[1]) == t
