"""Holstein chain workloads: model, Hamiltonian MPO, density MPOs, random MPS.

Site layout follows the reference's pp-Holstein mapping (holstein/input.h:138-149,
holstein/lattice.h:83-123): each molecule contributes one exciton site (dim 2)
followed, per vibrational mode, by a physical phonon site and an auxiliary site
(both dim ``cutoff``).  Phonon raising on the physical site is paired with
lowering on the auxiliary site, so the Hamiltonian conserves the U(1) charge
``N_ex + sum over modes of (n_phys + n_aux)`` (holstein/local.h:43-88).  The
auxiliary site starts at its maximum occupation (holstein/lattice.h:113-119), so
the physical subspace has ``n_phys + n_aux = cutoff - 1`` for every mode.

Hamiltonian (hbar = 1)::

    H = sum_i eps_i n_i + J sum_i (c_i^+ c_i+1 + c_i+1^+ c_i)
        + sum_ik omega_k b_ik^+ b_ik + sum_ik g_ik n_i (b_ik^+ A_ik^- + b_ik A_ik^+)

which is the operator the reference's ``totals`` builds (holstein/lattice.h:183-339)
from an input whose linear-coupling value is ``g * sqrt(2)`` (it multiplies the
value by sqrt(1/2), holstein/lattice.h:266).

The MPO is written directly as a finite-state machine with U(1)-labelled bond
states.  After removing unreachable states its bond sectors are those of the
reference's SVD-compressed ``Op/H_tot`` (e.g. ``[-1:1],[0:3],[1:1]`` after an
exciton site); both represent the same operator, which the tests check against
the reference-built MPO.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .kvio import BlockTensor

MPS_DIRS = (1, 1, -1)
MPO_DIRS = (1, 1, -1, -1)


@dataclass
class HolsteinChain:
    """A disordered Holstein chain of ``n_mol`` molecules.

    ``omega[k]`` is the frequency of mode k; ``g[i][k]`` the coupling of mode k on
    molecule i; ``eps[i]`` the site energy of molecule i; ``cutoff`` the local
    phonon dimension (occupations 0..cutoff-1, i.e. the reference's ``occ`` is
    ``cutoff - 1``).
    """

    n_mol: int
    omega: list
    g: list
    cutoff: int
    J: float = -1.0
    eps: list = None

    def __post_init__(self):
        if self.eps is None:
            self.eps = [0.0] * self.n_mol
        if len(self.g) != self.n_mol or any(len(r) != len(self.omega) for r in self.g):
            raise ValueError("g must be n_mol x n_modes")

    @property
    def n_modes(self) -> int:
        return len(self.omega)

    @property
    def occ(self) -> int:
        return self.cutoff - 1

    def site_types(self) -> list:
        """('e', i) / ('v', i, k) / ('a', i, k) per MPS site."""
        out = []
        for i in range(self.n_mol):
            out.append(("e", i))
            for k in range(self.n_modes):
                out.append(("v", i, k))
                out.append(("a", i, k))
        return out

    def site_dims(self) -> list:
        return [2 if t[0] == "e" else self.cutoff for t in self.site_types()]

    @property
    def n_sites(self) -> int:
        return self.n_mol * (1 + 2 * self.n_modes)

    @property
    def total_charge(self) -> int:
        return 1 + self.n_mol * self.n_modes * self.occ

    def exciton_sites(self) -> list:
        return [s for s, t in enumerate(self.site_types()) if t[0] == "e"]

    # ------------------------------------------------------------------ input
    def reference_input(self) -> str:
        """The same model as a reference text input for ``kln-holstein``
        (sections parsed by holstein/input.h:85-155)."""
        ne = self.n_mol
        lines = ["# electronic part"]
        terms = []
        for i in range(ne):
            if self.eps[i] != 0.0:
                terms.append((i + 1, i + 1, self.eps[i]))
        for i in range(ne - 1):
            terms.append((i + 1, i + 2, self.J))
            terms.append((i + 2, i + 1, self.J))
        lines.append(f"{ne} {len(terms)}")
        lines += [f"{a} {b} {v!r}" for a, b, v in terms]
        nv = ne * self.n_modes
        lines += ["", "# vibrational part", str(nv)]
        vib = 0
        lin = []
        order = []
        for i in range(ne):
            order.append(i)
            for k in range(self.n_modes):
                vib += 1
                lines.append(f"{vib} {self.omega[k]!r} {self.occ}")
                lin.append((vib, i + 1, i + 1, self.g[i][k] * math.sqrt(2.0)))
                order.append(vib + ne - 1)
        lines += ["", "# 1st-order coupling part", str(len(lin))]
        lines += [f"{v} {a} {b} {val!r}" for v, a, b, val in lin]
        lines += ["", "# 2nd-order coupling part", "0", "", "# reordering part",
                  " ".join(str(x) for x in order), ""]
        return "\n".join(lines)


# ---------------------------------------------------------------------- MPO
def _local_ops(d: int):
    """Dense local operators on a site of dimension d (rows = out state)."""
    eye = np.eye(d)
    raise_sqrt = np.zeros((d, d))
    raise_one = np.zeros((d, d))
    for n in range(d - 1):
        raise_sqrt[n + 1, n] = math.sqrt(n + 1.0)  # PhyRaise, holstein/local.h:43-50
        raise_one[n + 1, n] = 1.0  # AuxRaise, holstein/local.h:65-72
    return eye, raise_sqrt, raise_one


def _dense_to_blocks(W: np.ndarray, lq: list, rq: list) -> BlockTensor:
    """Cut W[s_out, wl, s_in, wr] into U(1) blocks (1, dim(ql), 1, dim(qr)).

    Physical states are their own charge sectors (charge = occupation).  Bond
    states are grouped by charge in ascending order."""
    d = W.shape[0]
    lsec = {}
    for idx, q in enumerate(lq):
        lsec.setdefault(q, []).append(idx)
    rsec = {}
    for idx, q in enumerate(rq):
        rsec.setdefault(q, []).append(idx)
    blocks = []
    for so in range(d):
        for si in range(d):
            for ql in sorted(lsec):
                qr = ql + so - si
                if qr not in rsec:
                    continue
                sub = W[so][np.ix_(lsec[ql], [si], rsec[qr])][:, 0, :]
                if not np.any(sub):
                    continue
                blk = sub.reshape(1, len(lsec[ql]), 1, len(rsec[qr])).astype(np.complex128)
                blocks.append(((so, ql, si, qr), blk))
    return BlockTensor(MPO_DIRS, blocks)


def _fsm_live(chain: HolsteinChain, terms) -> list:
    """Per bond, the FSM states reachable from 'I' at the left edge that can
    still reach 'F' at the right edge, in (charge, name) order."""
    types = chain.site_types()
    dims = chain.site_dims()
    ns = len(types)
    trans = [list(terms(s, types[s], dims[s])) for s in range(ns)]
    fwd = [set() for _ in range(ns + 1)]
    fwd[0] = {"I"}
    for s in range(ns):
        for a, b, op in trans[s]:
            if a in fwd[s] and np.any(op):
                fwd[s + 1].add(b)
    bwd = [set() for _ in range(ns + 1)]
    bwd[ns] = {"F"}
    for s in reversed(range(ns)):
        for a, b, op in trans[s]:
            if b in bwd[s + 1] and np.any(op):
                bwd[s].add(a)
    return [sorted(fwd[s] & bwd[s], key=lambda x: (_STATE_Q[x], _STATE_ORDER.index(x))) for s in range(ns + 1)]


def _fsm_dense(chain: HolsteinChain, terms, live: list, s: int) -> np.ndarray:
    """Site s of the FSM as a dense W[s_out, wl, s_in, wr] over the live states."""
    t, d = chain.site_types()[s], chain.site_dims()[s]
    L, R = live[s], live[s + 1]
    W = np.zeros((d, len(L), d, len(R)))
    for a, b, op in terms(s, t, d):
        if a in L and b in R:
            W[:, L.index(a), :, R.index(b)] += op
    return W


def _fsm_mpo(chain: HolsteinChain, terms):
    """Generic finite-state-machine MPO builder.

    ``terms(site, type)`` yields (from_state, to_state, dense local operator);
    states are named strings with a charge given by ``_STATE_Q``.  Unreachable
    states (not reachable from 'I' at the left edge, or unable to reach 'F' at
    the right edge) are pruned, then each site is cut into U(1) blocks."""
    live = _fsm_live(chain, terms)
    return [_dense_to_blocks(_fsm_dense(chain, terms, live, s), [_STATE_Q[x] for x in live[s]],
                             [_STATE_Q[x] for x in live[s + 1]]) for s in range(chain.n_sites)]


_STATE_Q = {"I": 0, "F": 0, "N": 0, "Cp": 1, "Cm": -1, "Bp": 1, "Bm": -1}
_STATE_ORDER = ["I", "N", "F", "Cp", "Bp", "Cm", "Bm"]


def _ham_terms(chain: HolsteinChain, coef):
    """The Holstein Hamiltonian's FSM transitions.  ``coef(kind, value, mode)``
    gives each transition's coefficient from its kind ("struct" for the
    identity pass-throughs and the operator strings, "eps", "J", "omega", "g"),
    its value in the Hamiltonian and, for omega and g, the mode index."""
    nm = chain.n_modes

    def terms(s, t, d):
        eye, bp, ap = _local_ops(d)
        bm, am = bp.T.copy(), ap.T.copy()
        n_e = np.diag([0.0, 1.0]) if d == 2 else None
        one = coef("struct", 1.0, None)
        # hopping states pass through phonon/aux sites only: at the next exciton
        # site they must terminate (nearest-neighbour hopping)
        for st in ("I", "F") if t[0] == "e" else ("I", "F", "Cp", "Cm"):
            yield st, st, one * eye
        if t[0] == "e":
            i = t[1]
            yield "I", "F", coef("eps", chain.eps[i], None) * n_e
            if i + 1 < chain.n_mol:
                yield "I", "Cp", one * bp  # c_i^+ (exciton: sqrt(1) = 1)
                yield "I", "Cm", one * bm  # c_i
            if i > 0:
                yield "Cp", "F", coef("J", chain.J, None) * bm  # J c_{i-1}^+ c_i
                yield "Cm", "F", coef("J", chain.J, None) * bp  # J c_i^+ c_{i-1}
            if nm > 0:
                yield "I", "N", one * n_e
        elif t[0] == "v":
            i, k = t[1], t[2]
            yield "I", "F", coef("omega", chain.omega[k], k) * (bp @ bm)
            yield "N", "Bp", coef("g", chain.g[i][k], k) * bp
            yield "N", "Bm", coef("g", chain.g[i][k], k) * bm
            if k + 1 < nm:
                yield "N", "N", one * eye
        else:  # aux site
            k = t[2]
            yield "Bp", "F", one * am
            yield "Bm", "F", one * ap
            if k + 1 < nm:
                yield "N", "N", one * eye

    return terms


def hamiltonian_mpo(chain: HolsteinChain) -> list:
    """The full Holstein Hamiltonian as an MPO (list of BlockTensor)."""
    return _fsm_mpo(chain, _ham_terms(chain, lambda kind, value, mode: value))


def hamiltonian_mpo_param(chain: HolsteinChain, names=("J", "omega", "g", "eps")) -> tuple:
    """The Hamiltonian as a parameter-linear MPO: (W, dW) with W the sites of
    hamiltonian_mpo(chain) and dW[name][s] the exact derivative of site s with
    respect to the parameter `name`, on the same block list as W[s] (zero
    blocks where the site does not depend on it).

    Every term of the Holstein Hamiltonian carries its coefficient on exactly
    one site tensor (J on the exciton site that closes a hop, eps on the
    exciton site, omega and g on the phonon site), so W_s is affine in the
    parameters and H is linear in them: W(theta') = W(theta) +
    sum_k (theta'_k - theta_k) dW_k, and dH/dtheta_k = sum_s (H with site s
    replaced by dW_k[s]).  This is the reference's direct-sum construction of
    H = sum_k theta_k H_k (Operator::operator+=, holstein/operator.h:54-70)
    without its truncation, so dW/dtheta is exact.  Names: "J"; "eps" (every
    molecule's site energy together); "omega" and "g" (every mode together)
    or "omega_k" / "g_k" (mode k: its frequency, or its coupling on every
    molecule)."""
    ham = _ham_terms(chain, lambda kind, value, mode: value)
    live = _fsm_live(chain, ham)
    W = _fsm_mpo(chain, ham)
    lq = [[_STATE_Q[x] for x in live[s]] for s in range(len(live))]
    dW = {}
    for name in names:
        terms = _ham_terms(chain, lambda kind, value, mode, name=name:
                           1.0 if (kind == name or (mode is not None and name == f"{kind}_{mode}")) else 0.0)
        dW[name] = [_blocks_like(W[s], _fsm_dense(chain, terms, live, s), lq[s], lq[s + 1])
                    for s in range(chain.n_sites)]
    return W, dW


def _blocks_like(template: BlockTensor, W: np.ndarray, lq: list, rq: list) -> BlockTensor:
    """Blocks of the dense W[s_out, wl, s_in, wr] on exactly the block list of
    `template` (same keys, order and shapes; zero blocks kept)."""
    lsec, rsec = {}, {}
    for idx, q in enumerate(lq):
        lsec.setdefault(q, []).append(idx)
    for idx, q in enumerate(rq):
        rsec.setdefault(q, []).append(idx)
    blocks = []
    for (so, ql, si, qr), blk in template.blocks:
        sub = W[so][np.ix_(lsec[ql], [si], rsec[qr])][:, 0, :]
        blocks.append(((so, ql, si, qr), sub.reshape(blk.shape).astype(np.complex128)))
    return BlockTensor(template.dirs, blocks)


def density_mpo(chain: HolsteinChain, site: int) -> list:
    """n_j on MPS site ``site`` (an exciton site) as a bond-dimension-1 MPO, the
    operator the reference's ``all_density`` writes to Op/Density_j
    (holstein/lattice.h:170-180)."""

    def terms(s, t, d):
        eye = np.eye(d)
        if s == site:
            yield "I", "F", np.diag([0.0, 1.0])
        else:
            yield "I", "I", eye
            yield "F", "F", eye

    return _fsm_mpo(chain, terms)


def identity_mpo(chain: HolsteinChain) -> list:
    def terms(s, t, d):
        if s == chain.n_sites - 1:
            yield "I", "F", np.eye(d)
        else:
            yield "I", "I", np.eye(d)

    return _fsm_mpo(chain, terms)


# ---------------------------------------------------------------- random MPS
def _bond_counts(chain: HolsteinChain):
    """Exact dimension of each bond charge sector in the physical subspace.

    Returns, per bond b = 0..ns (bond b is left of site b), two dicts
    charge -> number of left / right physical configurations."""
    types = chain.site_types()
    ns = len(types)
    occ = chain.occ
    Q = chain.total_charge
    # left: macro state (e_count, pending n_v or -1) -> multiplicity; charge computed
    left = []
    state = {(0, -1): 1}
    base = 0  # completed-mode charge so far
    n_e_seen = 0
    left.append({0: 1})
    for s in range(ns):
        t = types[s]
        new = {}
        if t[0] == "e":
            n_e_seen += 1
            for (ec, pend), m in state.items():
                new[(ec, pend)] = new.get((ec, pend), 0) + m
                if ec == 0:
                    new[(1, pend)] = new.get((1, pend), 0) + m
        elif t[0] == "v":
            for (ec, pend), m in state.items():
                for n in range(occ + 1):
                    new[(ec, n)] = new.get((ec, n), 0) + m
        else:
            for (ec, pend), m in state.items():
                new[(ec, -1)] = new.get((ec, -1), 0) + m
            base += occ
        state = new
        counts = {}
        for (ec, pend), m in state.items():
            q = ec + base + max(pend, 0)
            counts[q] = counts.get(q, 0) + m
        left.append(counts)
    # the exciton multiplicity: (1, .) states counted once per exciton site seen
    # is already handled by accumulating from ec==0 at each exciton site.
    right = [None] * (ns + 1)
    state = {(0, -1): 1}
    base = 0
    right[ns] = {Q: 1}  # keyed by LEFT charge of the bond: Q - right charge
    for s in reversed(range(ns)):
        t = types[s]
        new = {}
        if t[0] == "e":
            for (ec, pend), m in state.items():
                new[(ec, pend)] = new.get((ec, pend), 0) + m
                if ec == 0:
                    new[(1, pend)] = new.get((1, pend), 0) + m
        elif t[0] == "a":
            for (ec, pend), m in state.items():
                for n in range(occ + 1):  # n = n_aux; pending n_phys = occ - n
                    new[(ec, n)] = new.get((ec, n), 0) + m
        else:
            for (ec, pend), m in state.items():
                new[(ec, -1)] = new.get((ec, -1), 0) + m
            base += occ
        state = new
        counts = {}
        for (ec, pend), m in state.items():
            rq = ec + base + max(pend, 0)
            counts[Q - rq] = counts.get(Q - rq, 0) + m
        right[s] = counts
    return left, right


def random_mps_structure(chain: HolsteinChain, D: int) -> list:
    """Bond sector dimensions {charge: dim} for bonds 0..ns.

    Sector charges are those of the physical subspace reachable from both
    ends; D is shared among them in proportion to min(left, right) exact
    dimension, each sector capped by that minimum, then trimmed until every
    site's sector matrices can have full rank."""
    left, right = _bond_counts(chain)
    ns = chain.n_sites
    dims = chain.site_dims()
    bonds = []
    for b in range(ns + 1):
        cap = {q: min(left[b][q], right[b][q]) for q in left[b] if q in right[b]}
        cap = {q: c for q, c in cap.items() if c > 0}
        if b == 0 or b == ns:
            bonds.append({q: 1 for q in cap})
            continue
        tot = sum(min(c, D) for c in cap.values())
        alloc = {}
        if tot <= D:
            alloc = {q: min(c, D) for q, c in cap.items()}
        else:
            w = {q: min(c, D) for q, c in cap.items()}
            sw = float(sum(w.values()))
            alloc = {q: max(1, min(cap[q], int(math.floor(D * w[q] / sw)))) for q in cap}
            # distribute the remainder to the largest-weight sectors with room
            rem = D - sum(alloc.values())
            order = sorted(cap, key=lambda q: (-w[q], q))
            while rem > 0:
                progressed = False
                for q in order:
                    if rem == 0:
                        break
                    if alloc[q] < cap[q]:
                        alloc[q] += 1
                        rem -= 1
                        progressed = True
                if not progressed:
                    break
            while rem < 0:
                for q in sorted(alloc, key=lambda q: (alloc[q], q), reverse=True):
                    if rem == 0:
                        break
                    if alloc[q] > 1:
                        alloc[q] -= 1
                        rem += 1
        bonds.append(alloc)
    # full-rank trimming
    changed = True
    while changed:
        changed = False
        for s in range(ns):
            lb, rb = bonds[s], bonds[s + 1]
            for q in list(lb):
                cols = sum(rb.get(q + sg, 0) for sg in range(dims[s]))
                if lb[q] > cols:
                    lb[q] = cols
                    changed = True
                if lb[q] == 0:
                    del lb[q]
            for q in list(rb):
                rows = sum(lb.get(q - sg, 0) for sg in range(dims[s]))
                if rb[q] > rows:
                    rb[q] = rows
                    changed = True
                if rb[q] == 0:
                    del rb[q]
    return bonds


def random_mps(chain: HolsteinChain, D: int, seed: int) -> list:
    """Seeded random MPS in the physical charge sectors, right-canonical on
    sites 1..ns-1 with the normalised orthogonality centre on site 0 (the form
    TDVP::one_site / two_site start from, holstein/tdvp.h:78-141).

    Entries are re + i im with re, im ~ N(0, 1); each left-charge sector
    matrix of a site (rows D_l(q), columns the concatenated (sigma, D_r) blocks)
    is replaced by the orthonormal-row factor of its LQ decomposition and the
    triangular factor is carried into the site on the left (rescaled by its
    norm, which only changes the overall scale)."""
    rng = np.random.default_rng(seed)
    bonds = random_mps_structure(chain, D)
    dims = chain.site_dims()
    ns = chain.n_sites
    sites = []
    for s in range(ns):
        blocks = []
        for ql in sorted(bonds[s]):
            for sg in range(dims[s]):
                qr = ql + sg
                if qr in bonds[s + 1]:
                    sh = (bonds[s][ql], 1, bonds[s + 1][qr])
                    a = rng.standard_normal(sh) + 1j * rng.standard_normal(sh)
                    blocks.append(((ql, sg, qr), a))
        sites.append(BlockTensor(MPS_DIRS, blocks))
    for s in range(ns - 1, 0, -1):
        t = sites[s]
        by_left = {}
        for idx, (q, a) in enumerate(t.blocks):
            by_left.setdefault(q[0], []).append(idx)
        carry = {}
        for ql, idxs in by_left.items():
            mats = [t.blocks[i][1][:, 0, :] for i in idxs]
            M = np.concatenate(mats, axis=1)
            qh, rh = np.linalg.qr(M.conj().T)  # M^H = Q R  ->  M = R^H Q^H
            Lf = rh.conj().T
            Qm = qh.conj().T
            col = 0
            for i, m in zip(idxs, mats):
                w = m.shape[1]
                t.blocks[i] = (t.blocks[i][0], Qm[:, col:col + w].reshape(m.shape[0], 1, w).copy())
                col += w
            carry[ql] = Lf
        # the carried factors only set the overall scale (normalised at the
        # end); rescale them so long chains neither overflow nor underflow
        cn = np.sqrt(sum(np.vdot(x, x).real for x in carry.values()))
        carry = {q: x / cn for q, x in carry.items()}
        prev = sites[s - 1]
        prev.blocks = [(q, np.einsum("aib,bc->aic", a, carry[q[2]])) for q, a in prev.blocks]
    nrm = sites[0].norm()
    sites[0].blocks = [(q, a / nrm) for q, a in sites[0].blocks]
    return sites


# ---------------------------------------------------------- standard configs
def config_chain(name: str, seed: int = 0) -> tuple:
    """(chain, D, defaults) for the benchmark configurations, by name.

    holstein-1site-L8   L=8, one mode (omega=1, g=1), cutoff 8, D=32, 1TDVP
    holstein-2site-L32  L=32, two modes (0.2/0.5, 1.2/1.0), cutoff 16, D=128, 2TDVP
    holstein-2site-L64  L=64, four modes, cutoff 8, D=512, 2TDVP
    holstein-1site-L24  L=24, one mode, cutoff 12, D=96, 1TDVP
    """
    if name == "holstein-1site-L8":
        ch = HolsteinChain(8, [1.0], [[1.0]] * 8, cutoff=8)
        return ch, 32, dict(mode=1, steps=20, dt=0.05, max_iter=11, tol_exp=1e-8, tol_svd=1e-8)
    if name == "holstein-2site-L32":
        ch = HolsteinChain(32, [0.2, 1.2], [[0.5, 1.0]] * 32, cutoff=16)
        return ch, 128, dict(mode=2, steps=20, dt=0.05, max_iter=11, tol_exp=1e-8, tol_svd=1e-8)
    if name == "holstein-2site-L64":
        ch = HolsteinChain(64, [0.1, 0.4, 0.9, 1.5], [[0.3, 0.6, 0.8, 1.0]] * 64, cutoff=8)
        return ch, 512, dict(mode=2, steps=5, dt=0.05, max_iter=11, tol_exp=1e-8, tol_svd=1e-9)
    if name == "holstein-1site-L24":
        ch = HolsteinChain(24, [1.0], [[1.0]] * 24, cutoff=12)
        return ch, 96, dict(mode=1, steps=10, dt=0.05, max_iter=11, tol_exp=1e-8, tol_svd=0.0)
    raise KeyError(name)


def disordered_chain(index: int, seed: int = 1234) -> tuple:
    """One chain of the batched disordered ensemble: L uniform in [8, 48],
    D uniform in {32, 64, 128, 256}, eps ~ N(0, 0.5^2), omega = 1,
    g uniform in [0.5, 1.5], cutoff 8."""
    rng = np.random.default_rng(seed + index)
    L = int(rng.integers(8, 49))
    D = int(rng.choice([32, 64, 128, 256]))
    eps = list(rng.normal(0.0, 0.5, size=L))
    g = [[float(x)] for x in rng.uniform(0.5, 1.5, size=L)]
    return HolsteinChain(L, [1.0], g, cutoff=8, eps=eps), D
