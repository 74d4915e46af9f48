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
INC = [os.path.join(ROOT, "include"), "/usr/local/cuda/include"]


def test_mirror_header_compiles():
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    cmd = [gxx, "-std=c++14", "-fsyntax-only", *sum((["-I", i] for i in INC), []), SRC]
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
    r = subprocess.run([str(exe), *files, str(out), "12", "10", "8", repr(float(z["s_l"])),
                        repr(float(z["dt"])), "10"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    G = np.fromfile(out, dtype=np.float64).reshape(z["run10"].shape)
    assert np.array_equal(G, z["run10"])
    vol = float(r.stdout.split()[1])
    assert vol == pytest.approx(float(z["vol_run10"]), rel=1e-12)
