"""GPU parity: each hot-path primitive and whole TDVP trajectories of
libkvgpu (through the C ABI) against the reference's golden vectors and the
CPU restatement oracle.  FP64 path: agreement to rounding (1e-12 on
primitives, 1e-9 on observables over the trajectories)."""
import os

import numpy as np
import pytest

import kvtest_util as U

U.load_package()
O = U.load_oracle()
from kylin_v_gb300 import holstein as H  # noqa: E402
from kylin_v_gb300 import kvio  # noqa: E402

pytestmark = pytest.mark.gpu
G = U.GOLDEN
OPS = [(c, d) for c in ("tiny1", "tiny2m") for d in sorted(os.listdir(os.path.join(G, c))) if d.startswith("ops_site")]


@pytest.fixture(scope="module")
def gpu():
    from kylin_v_gb300 import kvgpu

    kvgpu.init(0)
    return kvgpu


def _load(case, d):
    mps, mpo = kvio.read_mps(f"{G}/{case}/in.mps"), kvio.read_mpo(f"{G}/{case}/H.mpo")
    rd = lambda n: kvio.read_kvt(f"{G}/{case}/{d}/{n}.kvt")  # noqa: E731
    return mps, mpo, rd, int(d[len("ops_site"):])


@pytest.mark.parametrize("case,d", OPS)
def test_contractions(gpu, case, d):
    mps, mpo, rd, i = _load(case, d)
    L, R, R2 = rd("envL"), rd("envR"), rd("envR2")
    A, B, W, W2 = mps[i], mps[i + 1], mpo[i], mpo[i + 1]
    tol = 1e-12
    assert U.tensor_diff(gpu.heff_apply(1, L, A, W, None, R).to_host(), rd("h1")) < tol
    mm = gpu.product(A, B, 1).to_host()
    assert U.tensor_diff(mm, rd("mm")) < tol
    assert U.tensor_diff(gpu.heff_apply(2, L, mm, W, W2, R2).to_host(), rd("h2")) < tol
    assert U.tensor_diff(gpu.heff_apply(0, rd("envL_next"), rd("svd21_V"), None, None, R).to_host(), rd("h0")) < tol
    assert U.tensor_diff(gpu.env_sweep(R, A, W, False).to_host(), rd("envR_prev")) < tol
    assert U.tensor_diff(gpu.env_sweep(L, rd("svd21_U"), W, True).to_host(), rd("envL_next")) < tol
    # scale argument
    h = gpu.heff_apply(1, L, A, W, None, R, scale=0.025).to_host()
    ref = rd("h1")
    ref.blocks = [(q, 0.025 * a) for q, a in ref.blocks]
    assert U.tensor_diff(h, ref) < tol


@pytest.mark.parametrize("case,d", OPS)
def test_lanczos_expm(gpu, case, d):
    mps, mpo, rd, i = _load(case, d)
    L, R, R2 = rd("envL"), rd("envR"), rd("envR2")
    A, W, W2 = mps[i], mpo[i], mpo[i + 1]
    k1, _ = gpu.local_krylov(1, L, A, W, None, R, 0.05, 11, 1e-8)
    assert U.tensor_diff(k1.to_host(), rd("k1")) < 1e-12
    k2, _ = gpu.local_krylov(2, L, rd("mm"), W, W2, R2, 0.05, 11, 1e-8)
    assert U.tensor_diff(k2.to_host(), rd("k2")) < 1e-12
    k0, _ = gpu.local_krylov(0, rd("envL_next"), rd("svd21_V"), None, None, R, 0.05, 11, 1e-8, reverse=True)
    assert U.tensor_diff(k0.to_host(), rd("k0")) < 1e-12
    # the same blocks as the reference's sum of Krylov vectors (no more, no fewer)
    for got, name in ((k1, "k1"), (k2, "k2"), (k0, "k0")):
        assert set(got.to_host().as_dict()) == set(rd(name).as_dict()), name
    # the Krylov dimension equals the oracle's
    _, it_o = O.local_krylov(1, L, A, W, None, R, 0.05, 11, 1e-8)
    _, it_g = gpu.local_krylov(1, L, A, W, None, R, 0.05, 11, 1e-8)
    assert it_o == it_g
    # a fixed-dimension run (tolerance 0) uses max_iter-1 vectors
    _, it_f = gpu.local_krylov(1, L, A, W, None, R, 0.05, 7, 0.0)
    assert it_f == 6


@pytest.mark.parametrize("case,d", OPS)
def test_svd(gpu, case, d):
    mps, mpo, rd, i = _load(case, d)
    D = U.manifest()[case]["D"]
    for name, src, r1, l2r in (("svd21", mps[i], 2, True), ("svd12", mps[i], 1, False),
                               ("svd22l", rd("mm"), 2, True), ("svd22r", rd("mm"), 2, False)):
        u, v, nk, nt = gpu.svd_impl(src, r1, l2r, 1e-8, D)
        uo, vo, so, nto = O.svd(src, r1, l2r, 1e-8, D)
        assert nk == len(so) and nt == nto
        assert U.tensor_diff(gpu.product(u, v, 1).to_host(), O.product(rd(name + "_U"), rd(name + "_V"), 1)) < 1e-12
        uh, vh = u.to_host(), v.to_host()
        assert uh.legs()[-1] == rd(name + "_U").legs()[-1]   # same kept sectors and dims
        # isometry: U^H U = 1 (l2r) / V V^H = 1 (r2l)
        iso = O.product(uh, uh, r1, O.OP_C, O.OP_N) if l2r else O.product(vh, vh, src.rank - r1, O.OP_N, O.OP_C)
        for q, a in iso.as_dict().items():
            assert np.abs(a - np.eye(a.shape[0])).max() < 1e-12


def _traj_case(case, ti):
    import sys

    sys.path.insert(0, G)
    import make_golden as MG

    ent = U.manifest()[case]
    ch = MG.cases()[case]["chain"]
    mps = H.random_mps(ch, ent["D"], seed=ent["seed"])
    return ch, mps, H.hamiltonian_mpo(ch), ent["trajectories"][ti]


# the FP64 path against every golden trajectory but the large mixed-only one
# (tests/test_gpu_mixed_trajectory.py runs that one on the mixed path)
FP64_CASES = sorted(c for c, e in U.manifest().items() if not e.get("mixed_only"))
TRAJ = [(c, i) for c in FP64_CASES for i in range(len(U.manifest()[c]["trajectories"]))]


@pytest.mark.parametrize("case,ti", TRAJ)
def test_tdvp_trajectory(gpu, case, ti):
    ch, mps, mpo, tr = _traj_case(case, ti)
    ref = U.read_traj(f"{G}/{case}/{tr['file']}")
    dens = [H.density_mpo(ch, j) for j in ch.exciton_sites()]
    ident = H.identity_mpo(ch)
    t = gpu.TDVP(mps, mpo, tr["tol_svd"], 1e-8, tr["maxD"], 11, 0.05)
    U.prepare_sa(t, case, tr)
    dmpo = [[gpu.Tensor.from_host(x) for x in d] for d in dens]
    hmpo = [gpu.Tensor.from_host(x) for x in mpo]
    imp = [gpu.Tensor.from_host(x) for x in ident]
    for k, mode in enumerate(U.stage_modes(tr["stage"])):
        t.sweep(mode)
        s = t.sites()
        assert abs(gpu.expectation(s, imp, s).real - ref[k][1]) < 1e-10
        assert abs(gpu.expectation(s, hmpo, s).real - ref[k][2]) < 1e-8
        pops = np.array([gpu.expectation(s, d, s).real for d in dmpo])
        assert np.abs(pops - ref[k][3:3 + len(dens)]).max() < 1e-9, k
        maxb = max(sum(x.to_host().legs()[2].values()) for x in s[:-1])
        assert maxb == int(ref[k][-1])


@pytest.mark.parametrize("case", FP64_CASES)
def test_sweep_reference_flops(gpu, case):
    """The flops a sweep credits (8*M*N*K over every zgemm the reference issues,
    Lanczos iterations as actually run) equal the oracle's count of its own
    zgemm calls for the same sweeps."""
    O = U.load_oracle()
    ch, mps, mpo, tr = _traj_case(case, 0)
    stg = [int(x) for x in tr["stage"].strip("[]").split(",")]
    mode = 2 if stg[1] else 1
    t = gpu.TDVP(mps, mpo, tr["tol_svd"], 1e-8, tr["maxD"], 11, 0.05)
    o = O.Tdvp(mps, mpo, tr["tol_svd"], 1e-8, tr["maxD"], 11, 0.05)
    for _ in range(2):
        O.flops(True)
        o.sweep(mode)
        of = O.flops(True)
        t.two_site() if mode == 2 else t.one_site()
        gf = t.stats()["ref_flops"]
        assert of > 0 and abs(gf - of) <= 1e-9 * of, (gf, of)


@pytest.mark.parametrize("case", FP64_CASES)
def test_canonicalize(gpu, case):
    """State::canonicalize on a non-canonical MPS: the state is unchanged,
    sites 1..ns-1 are right-orthonormal, and the bond dimensions equal those
    of the same SVD / product sequence run on the oracle."""
    O = U.load_oracle()
    ch, mps, _, _ = _traj_case(case, 0)
    rng = np.random.default_rng(5)
    bent = [kvio.BlockTensor(t.dirs, [(q, a * (1.0 + 0.3 * rng.standard_normal(a.shape))) for q, a in t.blocks])
            for t in mps]
    ident = [gpu.Tensor.from_host(x) for x in H.identity_mpo(ch)]
    out = gpu.canonicalize(bent)
    nin = gpu.expectation(bent, ident, bent).real
    assert abs(gpu.expectation(out, ident, out).real - nin) < 1e-10 * nin
    assert abs(gpu.expectation(out, ident, bent) - nin) < 1e-10 * nin
    host = [t.to_host() for t in out]
    for a in host[1:]:
        for _, blk in O.product(a, a, 2, O.OP_N, O.OP_C).as_dict().items():
            assert np.abs(blk - np.eye(blk.shape[0])).max() < 1e-12
    ref = list(bent)
    for i in range(len(ref) - 1):
        u, v, _, _ = O.svd(ref[i], 2, True, 0.0, 1000)
        ref[i], ref[i + 1] = u, O.product(v, ref[i + 1], 1)
    for i in range(len(ref) - 1, 0, -1):
        u, v, _, _ = O.svd(ref[i], 1, False, 0.0, 1000)
        ref[i], ref[i - 1] = v, O.product(ref[i - 1], u, 1)
    assert [t.legs()[2] for t in host[:-1]] == [t.legs()[2] for t in ref[:-1]]


@pytest.mark.parametrize("case", ["tiny1", "tiny2m"])
def test_global_krylov_then_tdvp_matches_oracle(gpu, case):
    """Global-Krylov steps followed by one- and two-site sweeps (the sweep
    environments rebuilt after the Krylov stage, in both) against the oracle."""
    ch, mps, mpo, tr = _traj_case(case, 0)
    D = tr["maxD"]
    dens = [H.density_mpo(ch, j) for j in ch.exciton_sites()]
    t = gpu.TDVP(mps, mpo, 1e-8, 1e-8, D, 11, 0.05)
    o = O.Tdvp(mps, mpo, 1e-8, 1e-8, D, 11, 0.05)
    dmpo = [[gpu.Tensor.from_host(x) for x in d] for d in dens]
    hmpo = [gpu.Tensor.from_host(x) for x in mpo]
    for mode in (0, 0, 2, 1):
        t.sweep(mode)
        o.sweep(mode)
        s, so = t.sites(), o.mps()
        assert abs(gpu.expectation(s, hmpo, s).real - O.join(so, mpo, so).real) < 1e-9, mode
        pops = np.array([gpu.expectation(s, d, s).real for d in dmpo])
        pref = np.array([O.join(so, d, so).real for d in dens])
        assert np.abs(pops - pref).max() < 1e-9, mode
