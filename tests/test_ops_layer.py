"""The reference's tensor-level C++ surface (include/holstein/kv_ops.h:
Tensor, Block, product, apply_*, env_sweep, local_krylov, svd_impl; and
State::canonicalize, Operator::join in kv_holstein.h) on the host side,
without a GPU.

tests/ops_layer_driver.cpp is written against the reference's header names.
It is compiled twice:

* against the real libkvgpu, to show the layer builds and links on the
  product library (it needs a GPU to run);
* against tests/kvgpu_oracle_double.cpp, a test double of the C ABI's entry
  points answered by the CPU oracle.  Run on each golden case, it checks the
  layer's own work: the upload and download of blocks, leg directions and
  charges, the operand modes, the Krylov exit record, the singular-value
  record (SVS) and the host-side tensor operations.  Its outputs are compared
  with the reference's dumps and with the oracle's answers.
"""
import json
import os
import subprocess

import numpy as np
import pytest

import kvtest_util as U

U.load_package()
O = U.load_oracle()
from kylin_v_gb300 import kvio  # noqa: E402

ROOT = U.ROOT
G = U.GOLDEN
CASES = [(c, d) for c in ("tiny1", "tiny2m") for d in sorted(os.listdir(os.path.join(G, c)))
         if d.startswith("ops_site")]
CXX = ["g++", "-std=c++17", "-O1", "-Wall", "-Wno-unused-function"]


@pytest.fixture(scope="module")
def double_driver(tmp_path_factory):
    """The driver linked against the oracle-backed test double of libkvgpu."""
    d = tmp_path_factory.mktemp("ops_layer")
    U.build_abi_double(d)
    subprocess.run(CXX + ["-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "ops_layer_driver.cpp"),
                          "-o", str(d / "ops_layer_driver"), f"-L{d}", "-lkvgpu", f"-Wl,-rpath,{d}"], check=True)
    return d / "ops_layer_driver"


def test_layer_builds_on_the_gpu_library(tmp_path):
    from kylin_v_gb300 import build

    lib_dir = os.path.dirname(build.build())
    subprocess.run(CXX + ["-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "ops_layer_driver.cpp"),
                          "-o", str(tmp_path / "drv"), f"-L{lib_dir}", "-lkvgpu", f"-Wl,-rpath,{lib_dir}"],
                   check=True)
    assert (tmp_path / "drv").exists()


def _svs_records(path):
    with open(path) as f:
        lines = [ln.strip() for ln in f if ln.strip()]
    recs, i = [], 0
    while i < len(lines):
        n = int(lines[i])
        recs.append([float(x) for x in lines[i + 1:i + 1 + max(n - 2, 0)]])
        i += 1 + max(n - 2, 0)
    return recs


@pytest.mark.parametrize("case,d", CASES)
def test_layer_matches_reference(double_driver, tmp_path, case, d):
    site = int(d[len("ops_site"):])
    D = U.manifest()[case]["D"]
    ops = os.path.join(G, case, d)
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([str(double_driver), os.path.join(G, case), ops, str(out), str(site), str(D)],
                       cwd=tmp_path, check=True, capture_output=True, text=True)
    info = json.loads(r.stdout.strip().splitlines()[-1])
    rd = lambda n: kvio.read_kvt(os.path.join(ops, n + ".kvt"))  # noqa: E731
    got = lambda n: kvio.read_kvt(str(out / (n + ".kvt")))  # noqa: E731

    # contractions and Krylov exponentials against the reference's dumps
    for name in ("h1", "envR_prev", "mm", "h2", "envL_next", "h0", "k1", "k2", "k0"):
        assert U.tensor_diff(got(name), rd(name)) < 1e-12, name
        assert got(name).dirs == rd(name).dirs, name
    # SVDs: singular vectors are unique up to a phase, so compare U.V
    for name in ("svd21", "svd12", "svd22l", "svd22r"):
        u, v = got(name + "_U"), got(name + "_V")
        assert u.dirs[-1] == -1 and v.dirs[0] == 1
        ref = O.product(rd(name + "_U"), rd(name + "_V"), 1)
        assert U.tensor_diff(O.product(u, v, 1), ref) < 1e-12, name

    # the Krylov exit records
    mps = kvio.read_mps(os.path.join(G, case, "in.mps"))
    mpo = kvio.read_mpo(os.path.join(G, case, "H.mpo"))
    L, R = rd("envL"), rd("envR")
    _, it1 = O.local_krylov(1, L, mps[site], mpo[site], None, R, 0.05, 11, 1e-8)
    _, it2 = O.local_krylov(2, L, rd("mm"), mpo[site], mpo[site + 1], rd("envR2"), 0.05, 11, 1e-8)
    _, it0 = O.local_krylov(0, rd("envL_next"), rd("svd21_V"), None, None, R, 0.05, 11, 1e-8, True)
    assert (info["k1_iters"], info["k2_iters"], info["k0_iters"]) == (it1, it2, it0)
    assert info["k1_maxitr"] == int(it1 >= 10)
    k1 = rd("k1")
    nk1 = np.sqrt(sum(np.vdot(a, a).real for _, a in k1.blocks))
    assert abs(info["k1_loss"] - (1.0 - nk1)) < 1e-12

    # the SVS records of the two two-site splits: kept count, then
    # log10(s_i s_{i-2} / s_{i-1}^2) of the kept values, largest first
    recs = _svs_records(tmp_path / "SVS")
    assert len(recs) == 2
    for rec, l2r in zip(recs, (True, False)):
        _, _, s, _ = O.svd(rd("mm"), 2, l2r, 1e-8, D)
        s = np.sort(s)[::-1]
        want = np.log10(s[2:] * s[:-2] / s[1:-1] ** 2)
        assert len(rec) == len(want)
        np.testing.assert_allclose(rec, want, rtol=0, atol=1e-9)

    # host-side tensor operations
    A = mps[site]
    nA2 = sum(np.vdot(a, a).real for _, a in A.blocks)
    assert abs(info["norm_A"] - np.sqrt(nA2)) < 1e-12
    assert abs(complex(info["overlap_re"], info["overlap_im"]) - (0.5 - 1j) * nA2) < 1e-12
    combo = kvio.BlockTensor(A.dirs, [(q, a * (0.5 + 1j)) for q, a in A.blocks])
    assert U.tensor_diff(got("A_combo"), combo) < 1e-14
    t210 = kvio.BlockTensor(tuple(reversed(A.dirs)),
                            [(tuple(reversed(q)), np.transpose(a, (2, 1, 0))) for q, a in A.blocks])
    assert got("A_t210").dirs == t210.dirs
    assert U.tensor_diff(got("A_t210"), t210) == 0.0
    # State::canonicalize and Operator::join: the canonical form holds the same
    # state (energy unchanged), every site right of the centre is
    # right-orthonormal, and the scalar products scale site 0
    j0, j1, j2 = (complex(info["join"][2 * k], info["join"][2 * k + 1]) for k in range(3))
    assert abs(j0 - O.join(mps, mpo, mps)) < 1e-12
    assert abs(j1 - j0) < 1e-10 * max(1.0, abs(j0))
    assert abs(j2 - j1) < 1e-12 * max(1.0, abs(j1))
    canon = [got(f"canon_{k}") for k in range(len(mps))]
    assert abs(O.join(canon, mpo, canon) - j1) < 1e-12
    for t in canon[1:]:
        rows = {}
        for q, a in t.blocks:
            rows.setdefault(q[0], []).append(a.reshape(a.shape[0], -1))
        for q, ms in rows.items():
            m = np.concatenate(ms, axis=1)
            np.testing.assert_allclose(m @ m.conj().T, np.eye(m.shape[0]), atol=1e-12)
    # State += and Operator += (direct sums): H + 2H is 3H, psi + psi is 2 psi,
    # and the summed legs carry both parts' dimensions per charge
    j3, j4 = (complex(info["join"][2 * k], info["join"][2 * k + 1]) for k in (3, 4))
    assert abs(j3 - 3 * j0) < 1e-10 * max(1.0, abs(j0))
    assert abs(j4 - 4 * j0) < 1e-10 * max(1.0, abs(j0))
    s1, m1 = got("sum_state_1"), got("sum_mpo_1")
    for leg in (0, 2):
        assert s1.legs()[leg] == {q: 2 * n for q, n in mps[1].legs()[leg].items()}
    for leg in (1, 3):
        assert m1.legs()[leg] == {q: 2 * n for q, n in mpo[1].legs()[leg].items()}
    assert U.tensor_diff(got("stack_1"), s1) == 0.0  # the tensor-level stack is the same direct sum
    # the two-leg bra/ket environment: identity on the first block's left sector
    q0, a0 = A.blocks[0]
    e = kvio.BlockTensor((1, -1), [((q0[0], q0[0]), np.eye(a0.shape[0], dtype=complex))])
    want = O.product(A, O.product(e, combo, 1), 2, O.OP_C, O.OP_N)
    assert U.tensor_diff(got("env2_l2r"), want) < 1e-12
