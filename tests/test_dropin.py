"""The drop-in C++ layer (include/holstein/): the reference's own driver
src/kln-tdvp.cpp compiles unchanged against it and, on a CPU test double of
the C ABI, runs the same trajectory as the reference built with its own
headers (CPU, where the reference tree is present); a driver using the same
calls reproduces the library's TDVP sweep on the GPU, checkpoint file
included."""
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


REF_BIN = os.path.join(ROOT, "oracle", "_ref", "kln-tdvp")


def _observables(case):
    """Norm, energy and site populations of an MPS on a golden case's chain."""
    import sys

    sys.path.insert(0, U.GOLDEN)
    import make_golden as MG  # noqa: E402

    from kylin_v_gb300 import holstein as H

    O = U.load_oracle()
    ch = MG.cases()[case]["chain"]
    mpo = kvio.read_mpo(os.path.join(U.GOLDEN, case, "H.mpo"))
    ident = H.identity_mpo(ch)
    dens = [H.density_mpo(ch, j) for j in ch.exciton_sites()]

    def obs(s):
        return np.array([O.join(s, ident, s).real, O.join(s, mpo, s).real] + [O.join(s, d, s).real for d in dens])

    return obs


@pytest.mark.skipif(not os.path.exists(REF_DRIVER) or not os.path.exists(REF_BIN) or _cxx() is None,
                    reason="reference tree, its compiled driver or g++ absent")
def test_reference_driver_runs_on_the_layer(tmp_path):
    """The reference's own src/kln-tdvp.cpp, unchanged, compiled against
    include/holstein/ and run on a CPU test double of the C ABI
    (tests/kvgpu_oracle_double.cpp), against the same driver compiled with
    the reference's own headers (oracle/_ref/kln-tdvp): two two-site and two
    one-site sweeps; every checkpoint has the same norm, energy, site
    populations and largest bond."""
    libdir = tmp_path / "lib"
    U.build_abi_double(libdir)
    (tmp_path / "src").mkdir()
    os.symlink(REF_DRIVER, tmp_path / "src" / "kln-tdvp.cpp")
    os.symlink(os.path.join(ROOT, "include", "holstein"), tmp_path / "holstein")
    exe = tmp_path / "kln-tdvp"
    r = subprocess.run([_cxx(), "-std=c++17", "-O1", str(tmp_path / "src" / "kln-tdvp.cpp"), "-o", str(exe),
                        f"-L{libdir}", "-lkvgpu", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    case = "tiny1"
    g = os.path.join(U.GOLDEN, case)
    D = U.manifest()[case]["D"]
    args = ["-w", os.path.join(g, "in.mps"), "-o", os.path.join(g, "H.mpo"), "-s", "[0,2,0,2]", "-v", "0.05",
            "-D", str(D), "-t", "1e-8"]
    runs = {}
    for name, prog in (("layer", str(exe)), ("reference", REF_BIN)):
        wd = tmp_path / name
        (wd / "State").mkdir(parents=True)  # the reference writes its checkpoints there, it does not create it
        r = subprocess.run([prog] + args, cwd=wd, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, name + ": " + r.stdout[-2000:] + r.stderr[-2000:]
        runs[name] = wd
    obs = _observables(case)
    for k in range(4):
        a = kvio.read_mps(str(runs["layer"] / "State" / f"T-{k}.mps"))
        b = kvio.read_mps(str(runs["reference"] / "State" / f"T-{k}.mps"))
        assert np.abs(obs(a) - obs(b)).max() < 1e-12, k
        assert [sum(t.legs()[2].values()) for t in a] == [sum(t.legs()[2].values()) for t in b], k


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


@pytest.mark.gpu
def test_dropin_sa_stage(tmp_path):
    """total_start with an SA-1TDVP stage through the C++ layer: the two-site
    sweeps write the SVS log, `nls.py` on PATH (this package's restatement of
    the reference's fit) writes beta, and the SA sweeps' checkpoints equal the
    library's own SA sweeps with those widths and the same seed.  The fitted
    widths match the ones the reference's fit wrote for the same chain."""
    exe = tmp_path / "dropin_driver"
    r = subprocess.run([_cxx(), "-std=c++17", "-O1", os.path.join(ROOT, "tests", "dropin_driver.cpp"),
                        "-I" + os.path.join(ROOT, "include"), "-o", str(exe), "-L" + LIBDIR, "-lkvgpu",
                        "-Wl,-rpath," + LIBDIR], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    import sys

    bindir = tmp_path / "bin"
    bindir.mkdir()
    fit = bindir / "nls.py"
    fit.write_text(f"#!/bin/sh\nexec {sys.executable} {os.path.join(ROOT, 'kylin-v_gb300', 'sa_fit.py')} \"$@\"\n")
    fit.chmod(0o755)
    g = U.GOLDEN
    tr = [t for t in U.manifest()["tiny1"]["trajectories"] if t["stage"] == "[0,2,2,0]"][0]
    mps_file, mpo_file = os.path.join(g, "tiny1", "in.mps"), os.path.join(g, "tiny1", "H.mpo")
    env = dict(os.environ, PATH=str(bindir) + os.pathsep + os.environ["PATH"], KV_SA_SEED=str(tr["sa_seed"]))
    r = subprocess.run([str(exe), mps_file, mpo_file, "[0,2,2,0]", str(tr["maxD"]), str(tr["tol_svd"])], cwd=tmp_path,
                       capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    widths = [float(x) for x in (tmp_path / "beta").read_text().split()]
    ref_widths = [float(x) for x in open(os.path.join(g, "tiny1", tr["beta"])).read().split()]
    np.testing.assert_allclose(widths, ref_widths, rtol=1e-6)
    from kylin_v_gb300 import kvgpu

    kvgpu.init(0)
    t = kvgpu.TDVP(kvio.read_mps(mps_file), kvio.read_mpo(mpo_file), tr["tol_svd"], 1e-8, tr["maxD"], 11, 0.05)
    t.set_sa([1.0 / float("{:21.15f}".format(w)) for w in widths], tr["sa_seed"])
    for k, mode in enumerate((2, 2, 3, 3)):
        t.sweep(mode)
        got = kvio.read_mps(str(tmp_path / "State" / f"T-{k}.mps"))
        want = [s.to_host() for s in t.sites()]
        assert len(got) == len(want)
        for a, b in zip(got, want):
            assert U.tensor_diff(a, b) < 1e-12
    assert t.sa_added() > 0
