"""The mixed-precision path over whole trajectories against the reference's
own golden trajectories (tests/golden, generated by the compiled reference in
complex128): the gate the benchmark metric names, max |dP_i(t)| <= 1e-6 over
every site population and step, and |dE(t)| <= 1e-6 |E|.

l32m3 is the two-site benchmark's local structure (two modes with omega
0.2 / 1.2 and g 0.5 / 1.0, cutoff 16, D = 128, SVD cutoff 1e-8) on three
molecules, 20 two-site steps at dt = 0.05; l64m2 the large single chain's
(four modes, cutoff 8, D = 512, SVD cutoff 1e-9) on two molecules, two
steps, with charge sectors up to 512 x 512; l8c8d32 is the one-site benchmark
(L = 8, cutoff 8, D = 32, 20 steps); tiny1 / tiny2m are the small one- and
two-site cases."""
import os

import numpy as np
import pytest

import kvtest_util as U

U.load_package()
from kylin_v_gb300 import holstein as H  # noqa: E402

pytestmark = pytest.mark.gpu
G = U.GOLDEN
POP_TOL = 1e-6   # max |P_i^mixed(t) - P_i^ref(t)| over sites and steps
ENERGY_TOL = 1e-6  # relative |E^mixed(t) - E^ref(t)| / |E^ref|

CASES = [(c, i) for c, e in U.manifest().items() for i, t in enumerate(e["trajectories"])
         if t["stage"].startswith("[0,")]  # one- and two-site stages (no global-Krylov step)


@pytest.fixture(scope="module")
def gpu():
    from kylin_v_gb300 import kvgpu

    kvgpu.init(0)
    return kvgpu


@pytest.mark.parametrize("case,ti", CASES)
def test_mixed_trajectory_within_population_gate(gpu, case, ti):
    import sys

    sys.path.insert(0, G)
    import make_golden as MG

    ent = U.manifest()[case]
    tr = ent["trajectories"][ti]
    ch = MG.cases()[case]["chain"]
    mps = H.random_mps(ch, ent["D"], seed=ent["seed"])
    mpo = H.hamiltonian_mpo(ch)
    ref = U.read_traj(os.path.join(G, case, tr["file"]))
    dens = [[gpu.Tensor.from_host(x) for x in H.density_mpo(ch, j)] for j in ch.exciton_sites()]
    hmpo = [gpu.Tensor.from_host(x) for x in mpo]
    t = gpu.TDVP(mps, mpo, tr["tol_svd"], 1e-8, tr["maxD"], 11, 0.05, gpu.KV_MIXED_3M_DIGITS)
    U.prepare_sa(t, case, tr)
    worst_p = worst_e = 0.0
    for k, mode in enumerate(U.stage_modes(tr["stage"])):
        t.sweep(mode)
        s = t.sites()
        pops = np.array([gpu.expectation(s, d, s).real for d in dens])
        e = gpu.expectation(s, hmpo, s).real
        worst_p = max(worst_p, float(np.abs(pops - ref[k][3:3 + len(dens)]).max()))
        worst_e = max(worst_e, abs(e - ref[k][2]) / abs(ref[k][2]))
        assert worst_p <= POP_TOL, (k, worst_p)
        assert worst_e <= ENERGY_TOL, (k, worst_e)
    print(f"{case} {tr['stage']}: max population error {worst_p:.2e}, max relative energy error {worst_e:.2e}")
