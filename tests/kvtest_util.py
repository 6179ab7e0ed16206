"""Shared helpers for the test-suite: package loading and tensor comparison."""
from __future__ import annotations

import importlib.util
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def load_package():
    if "kylin_v_gb300" not in sys.modules:
        d = os.path.join(ROOT, "kylin-v_gb300")
        spec = importlib.util.spec_from_file_location("kylin_v_gb300", os.path.join(d, "__init__.py"),
                                                      submodule_search_locations=[d])
        m = importlib.util.module_from_spec(spec)
        sys.modules["kylin_v_gb300"] = m
        spec.loader.exec_module(m)
    return sys.modules["kylin_v_gb300"]


def load_oracle():
    if os.path.join(ROOT, "oracle") not in sys.path:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # noqa: E402

    return oracle


def build_abi_double(dest) -> str:
    """Compile tests/kvgpu_oracle_double.cpp (the C ABI answered by the CPU
    oracle, for host-side tests of the C++ layer) into dest/libkvgpu.so."""
    import subprocess

    oracle_dir = os.path.dirname(load_oracle().build())
    os.makedirs(dest, exist_ok=True)
    so = os.path.join(str(dest), "libkvgpu.so")
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "kvgpu_oracle_double.cpp"), "-o", so, f"-L{oracle_dir}", "-lkvoracle",
                    f"-Wl,-rpath,{oracle_dir}"], check=True)
    return so


def manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


def tensor_diff(a, b) -> float:
    """Max abs difference of two block tensors compared block-by-block by
    (charges, shape); a block missing on one side counts as zeros."""
    da, db = a.as_dict(), b.as_dict()
    m = 0.0
    for k in set(da) | set(db):
        x = da.get(k)
        y = db.get(k)
        if x is None:
            m = max(m, float(np.abs(y).max(initial=0.0)))
        elif y is None:
            m = max(m, float(np.abs(x).max(initial=0.0)))
        else:
            m = max(m, float(np.abs(x - y).max(initial=0.0)))
    return m


def tensor_scale(a) -> float:
    return max((float(np.abs(x).max(initial=0.0)) for _, x in a.blocks), default=0.0)


def read_traj(path):
    rows = []
    with open(path) as f:
        for line in f:
            if line.startswith("#"):
                continue
            rows.append([float(x) for x in line.split()])
    return np.array(rows)


def stage_modes(stage: str) -> list:
    """Sweep modes of a total_start stage string [nK, n2TDVP, nSA, n1TDVP]
    (holstein/tdvp.h:297-385) in the order the driver runs them: 0 = one
    global-Krylov step, 2 = two_site, 3 = sa_site, 1 = one_site."""
    nk, n2, nsa, n1 = (int(x) for x in stage.strip("[]").split(","))
    return [0] * nk + [2] * n2 + [3] * nsa + [1] * n1


def sa_betas(case: str, tr: dict):
    """betaSet of a golden SA trajectory (holstein/tdvp.h:343-358): 1 / the
    value on every line longer than 3 characters of the beta file the
    reference's fit wrote; None for a trajectory without an SA stage."""
    if "beta" not in tr:
        return None
    with open(os.path.join(GOLDEN, case, tr["beta"])) as f:
        return [1.0 / float(line) for line in f if len(line.rstrip("\n")) > 3]


def prepare_sa(t, case: str, tr: dict):
    """Give a TDVP handle (GPU or oracle) the widths and seed of a golden SA
    trajectory; nothing for other trajectories."""
    b = sa_betas(case, tr)
    if b is not None:
        t.set_sa(b, tr["sa_seed"])
