"""The drop-in COCR_FP executable on broken calculation directories.

The reference's readers stop with a message when an input file cannot be
opened or read (Code/COCR_FP/For_Solvers.cpp:32-77, `Cannot_open_file` and
the short-read checks of HarmVect3d.cpp:181-229).  The drop-in does the same:
exit status 1 and a message naming the file, before any GPU work, so these
checks run on a machine without a GPU.
"""
import os
import subprocess

import pytest

from conftest import load_golden
from mtcalc_with_dfp_cocr_gb300 import slae_io


@pytest.fixture(scope="module")
def exe():
    from mtcalc_with_dfp_cocr_gb300 import build
    build.build()
    return build.EXE


def _case_dir(tmp_path):
    w, s, mesh, z1d, us, uc, v3, kit_iter, kit_r, nu, alfa = load_golden("small")
    d = str(tmp_path)
    w.mesh.write(d, nu=nu, alfa=alfa, eps=s.eps, maxiter=s.maxiter, receivers=w.receivers)
    slae_io.write_slae(d, s)
    return d


def _run(exe, d):
    return subprocess.run([exe], cwd=d, capture_output=True, text=True, timeout=120)


@pytest.mark.parametrize("name", ["ig", "gg", "pr", "kuslau", "xyz.dat", "nver.dat"])
def test_missing_file(exe, tmp_path, name):
    d = _case_dir(tmp_path)
    os.remove(os.path.join(d, name))
    r = _run(exe, d)
    assert r.returncode == 1
    assert name in r.stderr
    assert not os.path.exists(os.path.join(d, "v3.dat"))
    with open(os.path.join(d, "logharm3dCalc")) as f:
        assert "Error" in f.read()


@pytest.mark.parametrize("name", ["ig", "jg", "gg", "di", "pr"])
def test_truncated_file(exe, tmp_path, name):
    d = _case_dir(tmp_path)
    p = os.path.join(d, name)
    size = os.path.getsize(p)
    with open(p, "r+b") as f:
        f.truncate(size - 8)
    r = _run(exe, d)
    assert r.returncode == 1
    assert name in r.stderr
    assert not os.path.exists(os.path.join(d, "v3.dat"))


def test_kuslau_size_mismatch(exe, tmp_path):
    d = _case_dir(tmp_path)
    with open(os.path.join(d, "kuslau")) as f:
        t = f.read().split()
    with open(os.path.join(d, "kuslau"), "w") as f:
        f.write(f"{int(t[0]) + 2}\n{t[1]}\n{t[2]}\n")
    r = _run(exe, d)
    assert r.returncode == 1
    assert "kuslau" in r.stderr


def test_non_conforming_mesh_refused(exe, tmp_path):
    d = _case_dir(tmp_path)
    with open(os.path.join(d, "tsize3d.dat"), "w") as f:
        f.write("12\n")
    r = _run(exe, d)
    assert r.returncode == 1
    assert "non-conforming" in r.stderr
