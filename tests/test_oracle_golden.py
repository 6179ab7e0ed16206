"""The CPU restatement oracle against the reference's own outputs.

Golden vectors come from the compiled reference (tests/golden/make_golden.py):
block-level dumps of each hot-path primitive and per-sweep TDVP trajectories.
"""
import os

import numpy as np
import pytest

import kvtest_util as U

U.load_package()
O = U.load_oracle()
from kylin_v_gb300 import holstein as H  # noqa: E402
from kylin_v_gb300 import kvio  # noqa: E402

G = U.GOLDEN
OPS_CASES = [(c, d) for c in ("tiny1", "tiny2m") for d in sorted(os.listdir(os.path.join(G, c)))
             if d.startswith("ops_site")]


def _inputs(case):
    return kvio.read_mps(f"{G}/{case}/in.mps"), kvio.read_mpo(f"{G}/{case}/H.mpo")


@pytest.mark.parametrize("case,d", OPS_CASES)
def test_primitives_match_reference(case, d):
    mps, mpo = _inputs(case)
    i = int(d[len("ops_site"):])
    rd = lambda n: kvio.read_kvt(f"{G}/{case}/{d}/{n}.kvt")  # noqa: E731
    L, R, R2 = rd("envL"), rd("envR"), rd("envR2")
    A, B, W, W2 = mps[i], mps[i + 1], mpo[i], mpo[i + 1]
    tol = 1e-13
    assert U.tensor_diff(O.apply(1, L, A, W, None, R), rd("h1")) < tol
    assert U.tensor_diff(O.env_sweep(R, A, W, False), rd("envR_prev")) < tol
    mm = O.product(A, B, 1)
    assert U.tensor_diff(mm, rd("mm")) < tol
    assert U.tensor_diff(O.apply(2, L, mm, W, W2, R2), rd("h2")) < tol
    assert U.tensor_diff(O.env_sweep(L, rd("svd21_U"), W, True), rd("envL_next")) < tol
    assert U.tensor_diff(O.apply(0, rd("envL_next"), rd("svd21_V"), None, None, R), rd("h0")) < tol


@pytest.mark.parametrize("case,d", OPS_CASES)
def test_svd_and_krylov_match_reference(case, d):
    mps, mpo = _inputs(case)
    i = int(d[len("ops_site"):])
    rd = lambda n: kvio.read_kvt(f"{G}/{case}/{d}/{n}.kvt")  # noqa: E731
    L, R, R2 = rd("envL"), rd("envR"), rd("envR2")
    A, W, W2 = mps[i], mpo[i], mpo[i + 1]
    # singular vectors are unique up to a phase: compare the gauge-invariant U.V
    for name, src, r1, l2r in (("svd21", A, 2, True), ("svd12", A, 1, False),
                               ("svd22l", rd("mm"), 2, True), ("svd22r", rd("mm"), 2, False)):
        u, v, s, _ = O.svd(src, r1, l2r, 1e-8, U.manifest()[case]["D"])
        ref = O.product(rd(name + "_U"), rd(name + "_V"), 1)
        assert U.tensor_diff(O.product(u, v, 1), ref) < 1e-12
        assert sorted(len(x) for x in [u.legs()[-1]]) == sorted(len(x) for x in [rd(name + "_U").legs()[-1]])
    k1, _ = O.local_krylov(1, L, A, W, None, R, 0.05, 11, 1e-8)
    assert U.tensor_diff(k1, rd("k1")) < 1e-13
    k2, _ = O.local_krylov(2, L, rd("mm"), W, W2, R2, 0.05, 11, 1e-8)
    assert U.tensor_diff(k2, rd("k2")) < 1e-13
    k0, _ = O.local_krylov(0, rd("envL_next"), rd("svd21_V"), None, None, R, 0.05, 11, 1e-8, True)
    assert U.tensor_diff(k0, rd("k0")) < 1e-13


def _case_inputs(case, ent):
    import make_golden as MG  # noqa: E402  (tests/golden on sys.path below)

    ch = MG.cases()[case]["chain"]
    mps = H.random_mps(ch, ent["D"], seed=ent["seed"])
    n2 = [float(sum(np.vdot(a, a).real for _, a in t.blocks)) for t in mps]
    np.testing.assert_allclose(n2, ent["site_norms2"], rtol=1e-12)
    return ch, mps, H.hamiltonian_mpo(ch)


TRAJ = [(case, i) for case, ent in U.manifest().items() for i in range(len(ent["trajectories"]))]


@pytest.mark.parametrize("case,ti", TRAJ)
def test_tdvp_trajectory_matches_reference(case, ti):
    import sys

    sys.path.insert(0, G)
    ent = U.manifest()[case]
    tr = ent["trajectories"][ti]
    ch, mps, mpo = _case_inputs(case, ent)
    dens = [H.density_mpo(ch, j) for j in ch.exciton_sites()]
    ident = H.identity_mpo(ch)
    ref = U.read_traj(f"{G}/{case}/{tr['file']}")
    if ent["D"] >= 512:
        pytest.skip("D = 512: minutes per step on the CPU; the trajectory comes from the compiled reference and the "
                    "GPU gate test checks against it")
    t = O.Tdvp(mps, mpo, tr["tol_svd"], 1e-8, tr["maxD"], 11, 0.05)
    U.prepare_sa(t, case, tr)
    modes = U.stage_modes(tr["stage"])
    if ent.get("mixed_only"):
        modes = modes[:2]  # the D = 128 case: its first two steps (about 15 s a step here)
    for k, mode in enumerate(modes):
        t.sweep(mode)
        s = t.mps()
        assert abs(O.join(s, ident, s).real - ref[k][1]) < 1e-12
        assert abs(O.join(s, mpo, s).real - ref[k][2]) < 1e-11
        pops = np.array([O.join(s, d, s).real for d in dens])
        assert np.abs(pops - ref[k][3:3 + len(dens)]).max() < 1e-12
        maxb = max(sum(t_.legs()[2].values()) for t_ in s[:-1])
        assert maxb == int(ref[k][-1])


def test_own_mpo_equals_reference_hamiltonian():
    """<psi|H|psi> with this package's FSM MPO equals the reference-built Op/H_tot."""
    for case, ent in U.manifest().items():
        assert abs(ent["energy_ref_mpo"] - ent["energy_own_mpo"]) < 1e-9
    for case in ("tiny1", "tiny2m"):
        mps, mpo = _inputs(case)
        href = kvio.read_mpo(f"{G}/{case}/H_ref.mpo")
        assert abs(O.join(mps, mpo, mps) - O.join(mps, href, mps)) < 1e-12
