"""Generate the golden vectors in tests/golden/ from the compiled reference.

Run here (where the reference sources are mounted) with
``python tests/golden/make_golden.py`` (everything) or ``... --add`` (only the
trajectories the manifest lacks, from the committed inputs).  It builds the reference drivers and
the golden tools (oracle/Makefile, target ``ref``) and, for each case:

* writes the seeded inputs with this package's generators (Hamiltonian MPO,
  exciton-density MPOs, random right-canonical MPS) in the reference's binary
  formats, so the reference and the GPU library read identical bytes;
* runs ``kv_ref_ops`` (reference primitives on those inputs -> ``*.kvt``);
* runs ``kv_ref_tdvp`` (the reference TDVP driver, per-sweep norm / energy /
  populations / max bond -> ``traj_*.txt``);
* runs ``kln-holstein`` on the same model's text input and records
  <psi|H_ref|psi> so the MPO builder is pinned to the reference's own
  Hamiltonian construction.

Small cases keep every input and output; the config-sized case keeps only the
trajectory and an input checksum (its inputs are regenerated from the seed).
"""
from __future__ import annotations

import importlib.util
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_BIN = os.path.join(ROOT, "oracle", "_ref")


def _pkg():
    if "kylin_v_gb300" not in sys.modules:
        d = os.path.join(ROOT, "kylin-v_gb300")
        spec = importlib.util.spec_from_file_location("kylin_v_gb300", os.path.join(d, "__init__.py"),
                                                      submodule_search_locations=[d])
        m = importlib.util.module_from_spec(spec)
        sys.modules["kylin_v_gb300"] = m
        spec.loader.exec_module(m)
    return sys.modules["kylin_v_gb300"]


def cases():
    from kylin_v_gb300.holstein import HolsteinChain

    return {
        # 3 molecules x 1 mode, cutoff 4: 9 sites
        "tiny1": dict(chain=HolsteinChain(3, [1.0], [[1.0], [0.8], [1.2]], cutoff=4, eps=[0.1, -0.2, 0.3]),
                      D=8, seed=11, ops_sites=[1, 4], traj=[("[0,0,0,4]", 8, 1e-8), ("[0,3,0,0]", 8, 1e-8), ("[3,0,0,0]", 8, 1e-8),
                            ("[0,2,2,0]", 16, 1e-8)],
                      keep_inputs=True),
        # 2 molecules x 2 modes, cutoff 3: 10 sites
        "tiny2m": dict(chain=HolsteinChain(2, [1.0, 0.4], [[1.0, 0.6], [0.9, 0.5]], cutoff=3),
                       D=10, seed=12, ops_sites=[2, 6], traj=[("[0,0,0,3]", 10, 1e-8), ("[0,3,0,0]", 10, 1e-8),
                                                          ("[2,0,0,0]", 10, 1e-8), ("[0,2,2,0]", 20, 1e-8)],
                       keep_inputs=True),
        # the 1-site benchmark shape: L=8, 1 mode, cutoff 8, D=32, 20 steps
        "l8c8d32": dict(chain=HolsteinChain(8, [1.0], [[1.0]] * 8, cutoff=8), D=32, seed=1234, ops_sites=[7],
                        traj=[("[0,0,0,20]", 32, 1e-8)], keep_inputs=False),
        # the two-site benchmark's local structure (2 modes: omega 0.2 / 1.2, g 0.5 / 1.0, cutoff 16,
        # D = 128, SVD cutoff 1e-8) on 3 molecules (15 sites), 20 two-site steps: the trajectory the
        # mixed path's population gate is checked against (too slow for the FP64 trajectory tests)
        "l32m3": dict(chain=HolsteinChain(3, [0.2, 1.2], [[0.5, 1.0]] * 3, cutoff=16), D=128, seed=1234,
                      ops_sites=[], traj=[("[0,20,0,0]", 128, 1e-8)], keep_inputs=False, mixed_only=True),
        # the large single chain's local structure (4 modes: omega 0.1 / 0.4 / 0.9 / 1.5, g 0.3 / 0.6 /
        # 0.8 / 1.0, cutoff 8, D = 512, SVD cutoff 1e-9) on 2 molecules (18 sites), 2 two-site steps
        "l64m2": dict(chain=HolsteinChain(2, [0.1, 0.4, 0.9, 1.5], [[0.3, 0.6, 0.8, 1.0]] * 2, cutoff=8), D=512,
                      seed=1234, ops_sites=[], traj=[("[0,2,0,0]", 512, 1e-9)], keep_inputs=False, mixed_only=True),
    }


SA_SEED = 7  # seed of the SA stage's draws (oracle/shim/seeded_device.h)


def trajectory(ch, work, out, stage, maxd, tol, dens):
    """Run the reference TDVP driver on work/in.mps, work/H.mpo and write
    out/traj_<stage>.txt; returns the manifest entry.

    A stage with SA-1TDVP sweeps runs the driver built with the seeded
    random_device (kv_ref_tdvp_sa, KV_SA_SEED = SA_SEED) and the reference's
    own fit script bin/nls.py on PATH, as total_start calls it; the singular-
    value log it fits (SVS) and the widths it wrote (beta) are kept beside the
    trajectory."""
    for f in os.listdir(os.path.join(work, "State")):
        os.remove(os.path.join(work, "State", f))
    tag = stage.strip("[]").replace(",", "_")
    sa = int(stage.strip("[]").split(",")[2]) > 0
    env = None
    tool = "kv_ref_tdvp"
    if sa:
        tool = "kv_ref_tdvp_sa"
        ref = os.environ.get("KYLINV_REFERENCE", "/root/reference")
        wrap = os.path.join(work, "bin")
        os.makedirs(wrap, exist_ok=True)
        with open(os.path.join(wrap, "nls.py"), "w") as f:
            f.write(f"#!/bin/sh\nexec {sys.executable} {os.path.join(ref, 'bin', 'nls.py')} \"$@\"\n")
        os.chmod(os.path.join(wrap, "nls.py"), 0o755)
        env = dict(os.environ, PATH=wrap + os.pathsep + os.environ["PATH"], KV_SA_SEED=str(SA_SEED))
    txt = run([os.path.join(REF_BIN, tool), "-w", "in.mps", "-o", "H.mpo", "-s", stage,
               "-v", "0.05", "-D", str(maxd), "-t", str(tol), "-k", "11", "-e", "1e-8",
               "-d", ",".join(os.path.basename(p) for p in dens)], work, env)
    with open(os.path.join(out, f"traj_{tag}.txt"), "w") as f:
        f.write(f"# stage {stage} dt 0.05 maxD {maxd} tolSVD {tol} maxIter 11 tolExp 1e-8\n")
        f.write(txt)
    entry = {"stage": stage, "maxD": maxd, "tol_svd": tol, "file": f"traj_{tag}.txt"}
    if sa:
        shutil.copy(os.path.join(work, "beta"), os.path.join(out, f"beta_{tag}.txt"))
        shutil.copy(os.path.join(work, "SVS"), os.path.join(out, f"svs_{tag}.txt"))
        entry.update({"sa_seed": SA_SEED, "beta": f"beta_{tag}.txt", "svs": f"svs_{tag}.txt"})
    return entry


def add_missing_trajectories():
    """--add: the trajectories of cases() that the manifest lacks, from the
    committed inputs (the seeded generator is not bit-reproducible across BLAS
    thread counts, so existing vectors are left as they are)."""
    _pkg()
    from kylin_v_gb300 import holstein as H
    from kylin_v_gb300 import kvio

    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref", "-j4"], check=True,
                   stdout=subprocess.DEVNULL)
    with open(os.path.join(HERE, "manifest.json")) as f:
        manifest = json.load(f)
    for name, c in cases().items():
        if name not in manifest:
            manifest[name] = generate_case(name, c)
            continue
        have = {t["stage"] for t in manifest[name]["trajectories"]}
        todo = [t for t in c["traj"] if t[0] not in have]
        if not todo or not c["keep_inputs"]:
            continue
        ch = c["chain"]
        out = os.path.join(HERE, name)
        work = tempfile.mkdtemp(prefix="kvgold_")
        os.makedirs(os.path.join(work, "State"))
        for f in ("in.mps", "H.mpo"):
            shutil.copy(os.path.join(out, f), os.path.join(work, f))
        dens = []
        for j in ch.exciton_sites():
            p = os.path.join(work, f"D{j}.mpo")
            kvio.write_mpo(p, H.density_mpo(ch, j))
            dens.append(p)
        for stage, maxd, tol in todo:
            manifest[name]["trajectories"].append(trajectory(ch, work, out, stage, maxd, tol, dens))
        shutil.rmtree(work)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)


def run(cmd, cwd, env=None):
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError(f"{cmd}: {r.stdout}\n{r.stderr}")
    return r.stdout


def main():
    _pkg()
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref", "-j4"], check=True,
                   stdout=subprocess.DEVNULL)
    manifest = {name: generate_case(name, c) for name, c in cases().items()}
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)


def generate_case(name, c):
    """Inputs, primitive dumps and trajectories of one case; its manifest entry."""
    _pkg()
    from kylin_v_gb300 import holstein as H
    from kylin_v_gb300 import kvio

    ch = c["chain"]
    out = os.path.join(HERE, name)
    os.makedirs(out, exist_ok=True)
    work = tempfile.mkdtemp(prefix="kvgold_")
    os.makedirs(os.path.join(work, "State"))
    os.makedirs(os.path.join(work, "Op"))
    mps = H.random_mps(ch, c["D"], seed=c["seed"])
    mpo = H.hamiltonian_mpo(ch)
    kvio.write_mps(os.path.join(work, "in.mps"), mps)
    kvio.write_mpo(os.path.join(work, "H.mpo"), mpo)
    dens = []
    for j in ch.exciton_sites():
        p = os.path.join(work, f"D{j}.mpo")
        kvio.write_mpo(p, H.density_mpo(ch, j))
        dens.append(p)
    entry = {"D": c["D"], "seed": c["seed"], "n_sites": ch.n_sites,
             "site_norms2": [float(sum(np.vdot(a, a).real for _, a in t.blocks)) for t in mps]}
    # reference-built Hamiltonian on the same model
    with open(os.path.join(work, "chain.inp"), "w") as f:
        f.write(ch.reference_input())
    run([os.path.join(REF_BIN, "kln-holstein"), "-i", "chain.inp", "-t", "1e-14"], work)
    e_ref = run([os.path.join(REF_BIN, "kln-join"), "-a", "in.mps", "-b", "in.mps", "-o", "Op/H_tot"], work)
    e_mine = run([os.path.join(REF_BIN, "kln-join"), "-a", "in.mps", "-b", "in.mps", "-o", "H.mpo"], work)
    entry["energy_ref_mpo"] = float(e_ref.strip().strip("()").split(",")[0])
    entry["energy_own_mpo"] = float(e_mine.strip().strip("()").split(",")[0])
    if c["keep_inputs"]:
        for f in ("in.mps", "H.mpo"):
            shutil.copy(os.path.join(work, f), os.path.join(out, f))
        shutil.copy(os.path.join(work, "Op", "H_tot"), os.path.join(out, "H_ref.mpo"))
        for site in c["ops_sites"]:
            od = os.path.join(out, f"ops_site{site}")
            os.makedirs(od, exist_ok=True)
            run([os.path.join(REF_BIN, "kv_ref_ops"), "-w", "in.mps", "-o", "H.mpo", "-i", str(site),
                 "-v", "0.05", "-k", "11", "-e", "1e-8", "-t", "1e-8", "-D", str(c["D"]), "-O", od], work)
    entry["trajectories"] = [trajectory(ch, work, out, stage, maxd, tol, dens) for stage, maxd, tol in c["traj"]]
    if c.get("mixed_only"):
        entry["mixed_only"] = True
    shutil.rmtree(work)
    return entry


if __name__ == "__main__":
    add_missing_trajectories() if "--add" in sys.argv[1:] else main()
