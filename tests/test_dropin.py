"""The drop-in C++ layer (include/holstein/): the reference's own driver
src/kln-tdvp.cpp compiles unchanged against it (CPU, where the reference tree
is present), and a driver using the same calls reproduces the library's TDVP
sweep on the GPU, checkpoint file included."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import kvtest_util as U

U.load_package()
from kylin_v_gb300 import kvio  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "kylin-v_gb300", "_build")
REF_DRIVER = os.path.join(os.environ.get("KYLINV_REFERENCE", "/root/reference"), "src", "kln-tdvp.cpp")


def _cxx():
    return shutil.which("g++")


@pytest.mark.skipif(not os.path.exists(REF_DRIVER) or _cxx() is None, reason="reference tree or g++ absent")
def test_reference_driver_compiles_unchanged(tmp_path):
    # src/kln-tdvp.cpp includes "../holstein/tdvp.h": a symlink farm puts the
    # drop-in headers at that relative path without copying the driver
    (tmp_path / "src").mkdir()
    os.symlink(REF_DRIVER, tmp_path / "src" / "kln-tdvp.cpp")
    os.symlink(os.path.join(ROOT, "include", "holstein"), tmp_path / "holstein")
    lib = os.path.join(LIBDIR, "libkvgpu.so")
    if not os.path.exists(lib):
        pytest.skip("libkvgpu.so not built")
    r = subprocess.run([_cxx(), "-std=c++17", str(tmp_path / "src" / "kln-tdvp.cpp"), "-o", str(tmp_path / "kln-tdvp"),
                        "-L" + LIBDIR, "-lkvgpu", "-Wl,-rpath," + LIBDIR], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


@pytest.mark.gpu
def test_dropin_driver_matches_library(tmp_path):
    exe = tmp_path / "dropin_driver"
    r = subprocess.run([_cxx(), "-std=c++17", "-O1", os.path.join(ROOT, "tests", "dropin_driver.cpp"),
                        "-I" + os.path.join(ROOT, "include"), "-o", str(exe), "-L" + LIBDIR, "-lkvgpu",
                        "-Wl,-rpath," + LIBDIR], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    g = U.GOLDEN
    D = U.manifest()["tiny2m"]["D"]
    mps_file, mpo_file = os.path.join(g, "tiny2m", "in.mps"), os.path.join(g, "tiny2m", "H.mpo")
    r = subprocess.run([str(exe), mps_file, mpo_file, "[1,1,0,1]", str(D), "1e-8"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "Max bond dimension" in r.stdout
    from kylin_v_gb300 import kvgpu

    kvgpu.init(0)
    t = kvgpu.TDVP(kvio.read_mps(mps_file), kvio.read_mpo(mpo_file), 1e-8, 1e-8, D, 11, 0.05)
    for k, sweep in enumerate((t.global_krylov, t.two_site, t.one_site)):
        sweep()
        got = kvio.read_mps(str(tmp_path / "State" / f"T-{k}.mps"))
        want = [s.to_host() for s in t.sites()]
        assert len(got) == len(want)
        for a, b in zip(got, want):
            assert U.tensor_diff(a, b) < 1e-12
