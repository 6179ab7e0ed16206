"""The SA-1TDVP stage's width fit (kylin-v_gb300/sa_fit.py) against the widths
the reference's own fit script (bin/nls.py) wrote from the same singular-value
log, in the seeded reference runs that made the golden SA trajectories."""
import os

import numpy as np
import pytest

import kvtest_util as U

U.load_package()
from kylin_v_gb300 import sa_fit  # noqa: E402

SA = [(c, t) for c, e in U.manifest().items() for t in e["trajectories"] if "beta" in t]


@pytest.mark.parametrize("case,tr", SA, ids=[f"{c}-{t['stage']}" for c, t in SA])
def test_widths_match_reference_fit(case, tr, tmp_path):
    svs = os.path.join(U.GOLDEN, case, tr["svs"])
    per_bond = sa_fit.read_svs(svs)
    ref = [float(x) for x in open(os.path.join(U.GOLDEN, case, tr["beta"])).read().split()]
    assert len(per_bond) == len(ref)  # one width per bond
    got = sa_fit.fit_widths(per_bond)
    np.testing.assert_allclose(got, ref, rtol=1e-9)
    # the script form writes the file the drop-in layer reads
    out = tmp_path / "beta"
    assert sa_fit.main([svs, str(out)]) == 0
    np.testing.assert_allclose([float(x) for x in out.read_text().split()], ref, rtol=1e-9)


def test_short_bonds_get_unit_width():
    assert sa_fit.fit_widths([[0.1, -0.2], []]) == [1.0, 1.0]
