"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public dataset is involved: every structure and parameter set here is generated
from a seed (20261203 + config id) following the recipe of the five configurations:

* residue types uniform over 20; each chain a self-avoiding C-alpha walk with 3.8 A
  bonds confined to a sphere of radius 12 A x (n/76)^(1/3) (compact globule);
* contact energies: symmetric 20x20 epsilon ~ U[-1.2, 0.4] kcal/mol, stored as the
  reference's raw table value e = epsilon / (lambda RT) + e0 so that
  lambda (e - e0) RT = epsilon (src/Potential.cpp:14 and :187-201);
* vdW radius sigma_type ~ U[4.5, 7.0] A (sigma_ij = mean), charge +1 on 12 % and -1
  on 12 % of residues;
* cubic periodic box, Debye length 10 A, dielectric 80 (the reference constants).

c0  plain REMC: 2 rigid chains of 76, box 150 A, 20 replicas 288-450 K
c1  flexible linker: 76 + 10 + 76 residues in one chain, residues 75..86 joined by a
    flexible segment, seeded 20x20x4 torsion table, 32 replicas, flex moves 30 %
c2  crowded: 24 proteins of U[60,160] residues + 40 crowders of 20 residues
    (repulsive epsilon = +0.1 kcal/mol with everything, uncharged), box 250 A,
    32 replicas
c3  batched uneven: 96 simulations, 2-12 molecules, lengths log-U[40,400], 8-40 replicas
c4  8 copies of c0's protein in a 120 A box, 32 replicas
"""
import math

import numpy as np

LAMBDA = np.float32(0.159)
E0 = np.float32(-2.27)
RT = np.float32(0.59218674898147583)
BOND = 3.8
CROWDER_TYPE = 20


class Molecule:
    def __init__(self, xyz, types, charges, radii, segments=(), all_flexible=False, crowder=False,
                 chain_ids=None, res_seq=None):
        n = len(types)
        self.xyz = np.ascontiguousarray(xyz, np.float32).reshape(n, 3)
        self.types = np.ascontiguousarray(types, np.int32)
        self.charges = np.ascontiguousarray(charges, np.float32)
        self.radii = np.ascontiguousarray(radii, np.float32)
        self.segments = [list(map(int, s)) for s in segments]
        self.all_flexible = bool(all_flexible)
        self.crowder = bool(crowder)
        self.chain_ids = chain_ids if chain_ids is not None else ["A"] * n
        self.res_seq = np.ascontiguousarray(res_seq if res_seq is not None else np.arange(1, n + 1), np.int32)
        self.chain_index = np.zeros(n, np.int32)

    @property
    def n(self):
        return len(self.types)


class Simulation:
    def __init__(self, molecules, box, temperatures, translate_steps, rotate_steps, move_weights=(1, 1, 1, 1),
                 rigid_rotate_prob=0.5, repulsive_crowding=False):
        self.molecules = molecules
        self.repulsive_crowding = bool(repulsive_crowding)
        self.box = float(box)
        self.temperatures = np.ascontiguousarray(temperatures, np.float32)
        self.translate_steps = np.ascontiguousarray(translate_steps, np.float32)
        self.rotate_steps = np.ascontiguousarray(rotate_steps, np.float64)
        self.move_weights = tuple(float(w) for w in move_weights)
        self.rigid_rotate_prob = float(rigid_rotate_prob)

    @property
    def n_residues(self):
        return sum(m.n for m in self.molecules)


class Workload:
    def __init__(self, name, sims, lj_raw, torsion_V=None, torsion_phase=None, seed=0, notes=""):
        self.name = name
        self.sims = sims
        self.lj_raw = np.ascontiguousarray(lj_raw, np.float32)
        self.ntypes = self.lj_raw.shape[0]
        self.torsion_V = torsion_V
        self.torsion_phase = torsion_phase
        self.seed = seed
        self.notes = notes

    @property
    def n_replicas(self):
        return sum(len(s.temperatures) for s in self.sims)


def ladder(lo, hi, n):
    """Geometric ladder as Simulation::init forms it (src/Simulation.cpp:590-598)."""
    if n == 1:
        return np.array([lo], np.float64)
    g = (hi / lo) ** (1.0 / (n - 1))
    return np.array([lo * g ** i for i in range(n)], np.float64)


def raw_from_epsilon(eps_kcal):
    """Reference raw table value with lambda (e - e0) RT == eps (float arithmetic)."""
    eps = np.asarray(eps_kcal, np.float32)
    return (eps / (LAMBDA * RT) + E0).astype(np.float32)


def contact_table(rng, ntypes=20, with_crowder=False, crowder_eps=0.1):
    eps = rng.uniform(-1.2, 0.4, size=(ntypes, ntypes)).astype(np.float32)
    eps = np.triu(eps) + np.triu(eps, 1).T
    if with_crowder:
        full = np.full((ntypes + 1, ntypes + 1), crowder_eps, np.float32)
        full[:ntypes, :ntypes] = eps
        eps = full
    return raw_from_epsilon(eps)


def _norm3(v):
    """Euclidean length of a 3-vector in plain IEEE double arithmetic.  The generator
    avoids BLAS (np.linalg.norm, @) so that a seed gives the same structures on every
    CPU architecture and numpy build."""
    x, y, z = float(v[0]), float(v[1]), float(v[2])
    return math.sqrt(x * x + y * y + z * z)


def _min_d2(P, k, p):
    """Smallest squared distance from p to rows 0..k-1 of P (elementwise arithmetic)."""
    if k <= 0:
        return 1e18
    dx = P[:k, 0] - p[0]
    dy = P[:k, 1] - p[1]
    dz = P[:k, 2] - p[2]
    return float((dx * dx + dy * dy + dz * dz).min())


def _centre(P):
    c = [math.fsum(P[:, j].tolist()) / len(P) for j in range(3)]
    return P - np.array(c)


def _apply(X, R):
    """Rows of X rotated by R (X @ R.T written out elementwise)."""
    return X[:, 0:1] * R[:, 0] + X[:, 1:2] * R[:, 1] + X[:, 2:3] * R[:, 2]


def _mat3(A, B):
    return A[:, 0:1] * B[0:1, :] + A[:, 1:2] * B[1:2, :] + A[:, 2:3] * B[2:3, :]


def _unit_step(rng, length, bias=None, spread=1.0):
    d = rng.normal(size=3) * spread
    if bias is not None:
        d = d + bias
    return d * (length / _norm3(d))


def _first_free(P, k, cand, r_max, min_sep):
    """Index of the first row of cand within r_max of the origin and at least min_sep
    from rows 0..k-1 of P, or -1 (elementwise arithmetic throughout)."""
    ok = cand[:, 0] * cand[:, 0] + cand[:, 1] * cand[:, 1] + cand[:, 2] * cand[:, 2] <= r_max * r_max
    if k > 0:
        dx = P[:k, 0][None, :] - cand[:, 0:1]
        dy = P[:k, 1][None, :] - cand[:, 1:2]
        dz = P[:k, 2][None, :] - cand[:, 2:3]
        ok &= (dx * dx + dy * dy + dz * dz).min(1) >= min_sep * min_sep
    idx = np.flatnonzero(ok)
    return int(idx[0]) if len(idx) else -1


def compact_chain(rng, n, radius=None, min_sep=4.0, tries=320, block=16):
    """Self-avoiding walk of n residues, 3.8 A bonds, inside a sphere; centred on 0.
    Each step draws candidate bond directions `block` at a time and keeps the first
    one that stays in the sphere and clear of the chain."""
    if radius is None:
        radius = 12.0 * (n / 76.0) ** (1.0 / 3.0)
    P = np.zeros((n, 3))
    for attempt in range(100):
        if attempt % 5 == 4:  # long chains jam in the sphere: loosen it a little
            radius *= 1.08
        ok = True
        for k in range(1, n):
            for _t in range(0, tries, block):
                d = rng.normal(size=(block, 3))
                nrm = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
                cand = P[k - 1] + d * (BOND / nrm)[:, None]
                j = _first_free(P, k - 1, cand, radius, min_sep)
                if j >= 0:
                    P[k] = cand[j]
                    break
            else:
                ok = False
                break
        if ok:
            return _centre(P).astype(np.float32)
    raise RuntimeError("could not grow a compact chain of %d residues" % n)


def two_domain_linker(rng, na, nl, nb, clearance=6.0, min_sep=4.0):
    """Domain a, a self-avoiding linker of nl residues grown outward from a's last
    residue, then domain b attached at the linker's end and turned away from a.
    Residues four or more apart along the chain (the pairs that interact) keep
    `clearance` between them; residues two or three apart keep `min_sep`."""
    c2, s2 = clearance * clearance, min_sep * min_sep

    def clear(P, k_end, i, p):
        # candidate p at chain index i against rows 0..k_end-1 (chain indices 0..k_end-1)
        far = min(i - 3, k_end)
        if _min_d2(P, far, p) < c2:
            return False
        lo, hi = max(i - 3, 0), min(i - 1, k_end)
        return hi <= lo or _min_d2(P[lo:], hi - lo, p) >= s2

    for _ in range(200):
        a = compact_chain(rng, na).astype(np.float64)
        out = a[-1] / (_norm3(a[-1]) + 1e-9)
        P = np.zeros((na + nl, 3))
        P[:na] = a
        k = na
        ok = True
        for _l in range(nl):
            for _t in range(500):
                p = P[k - 1] + _unit_step(rng, BOND, bias=out, spread=0.7)
                if clear(P, k, k, p):
                    P[k] = p
                    k += 1
                    break
            else:
                ok = False
                break
        if not ok:
            continue
        b = compact_chain(rng, nb).astype(np.float64)
        head = P[k - 1].copy()
        for _t in range(500):
            u = out + 0.5 * rng.normal(size=3)
            u = u / _norm3(u)
            R = rotation_between(-b[0], u)
            Q = rotation_between(np.array([1.0, 0, 0]), rng.normal(size=3))  # spin about the axis
            bb = _apply(_apply(b - b[0], Q), R)
            bb = bb - bb[0] + head + BOND * u
            if all(clear(P, k, k + t, q) for t, q in enumerate(bb)) and _norm3(bb[0] - head) > 3.7:
                return np.concatenate([P, bb]).astype(np.float32)
    raise RuntimeError("could not build the two-domain linker structure")


def rotation_between(v1, v2):
    """Rotation matrix taking direction v1 onto direction v2 (Rodrigues)."""
    a = np.asarray(v1, np.float64) / _norm3(v1)
    b = np.asarray(v2, np.float64) / _norm3(v2)
    v = np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]])
    c = float(a[0] * b[0] + a[1] * b[1] + a[2] * b[2])
    if _norm3(v) < 1e-12:
        return np.eye(3) if c > 0 else -np.eye(3)
    K = np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])
    return np.eye(3) + K + _mat3(K, K) * (1.0 / (1.0 + c))


def residue_params(rng, n, sigma_type, charged=True):
    types = rng.integers(0, 20, size=n).astype(np.int32)
    u = rng.random(n)
    charges = np.where(u < 0.12, 1.0, np.where(u < 0.24, -1.0, 0.0)).astype(np.float32) if charged \
        else np.zeros(n, np.float32)
    radii = sigma_type[types].astype(np.float32)
    return types, charges, radii


def place_centres(rng, radii, box, tries=10000):
    """Non-overlapping centres in the box (minimum image), largest first."""
    order = np.argsort(-np.asarray(radii), kind="stable")
    centres = [None] * len(radii)
    C = np.zeros((len(radii), 3))
    rad = np.zeros(len(radii))
    k = 0
    for i in order:
        for _ in range(tries):
            c = rng.uniform(0, box, 3)
            if k:
                d = C[:k] - c
                d = d - box * np.round(d / box)
                d2 = d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2]
                lim = rad[:k] + radii[i] + 4.0
                if np.any(d2 < lim * lim):
                    continue
            centres[i] = c
            C[k], rad[k] = c, radii[i]
            k += 1
            break
        else:
            raise RuntimeError("could not place molecule %d" % i)
    return centres


def protein(rng, n, sigma_type, centre):
    xyz = compact_chain(rng, n) + np.asarray(centre, np.float32)
    t, q, s = residue_params(rng, n, sigma_type)
    return Molecule(xyz, t, q, s)


def rigid_sim(rng, lengths, box, n_rep, sigma_type, crowders=0, crowder_len=20, t_lo=288.0, t_hi=450.0,
              tr=(0.5, 2.0), rot=(0.2, 0.2)):
    rad = [12.0 * (n / 76.0) ** (1.0 / 3.0) for n in lengths] + [12.0 * (crowder_len / 76.0) ** (1 / 3)] * crowders
    centres = place_centres(rng, rad, box)
    mols = [protein(rng, n, sigma_type, centres[k]) for k, n in enumerate(lengths)]
    for k in range(crowders):
        xyz = compact_chain(rng, crowder_len) + np.asarray(centres[len(lengths) + k], np.float32)
        mols.append(Molecule(xyz, np.full(crowder_len, CROWDER_TYPE, np.int32), np.zeros(crowder_len, np.float32),
                             np.full(crowder_len, 5.0, np.float32), crowder=True))
    return Simulation(mols, box, ladder(t_lo, t_hi, n_rep), ladder(tr[0], tr[1], n_rep),
                      ladder(rot[0], rot[1], n_rep))


def make(config, seed=None):
    """The workload of configuration c0..c4."""
    cid = int(str(config).lstrip("c"))
    seed = 20261203 + cid if seed is None else seed
    rng = np.random.default_rng(seed)
    sigma_type = rng.uniform(4.5, 7.0, size=21).astype(np.float32)
    if cid == 0:
        table = contact_table(rng)
        sim = rigid_sim(rng, [76, 76], 150.0, 20, sigma_type)
        return Workload("c0: 2x76 rigid, box 150 A, 20 replicas", [sim], table, seed=seed)
    if cid == 1:
        table = contact_table(rng)
        V = rng.uniform(0.0, 1.5, size=(20, 20, 4))
        S = rng.uniform(0.0, 2 * math.pi, size=(20, 20, 4))
        xyz = two_domain_linker(rng, 76, 10, 76) + np.float32(75.0)
        t, q, s = residue_params(rng, 162, sigma_type)
        mol = Molecule(xyz, t, q, s, segments=[list(range(75, 87))])
        sim = Simulation([mol], 150.0, ladder(288.0, 450.0, 32), ladder(0.5, 2.0, 32), ladder(0.2, 0.2, 32),
                         move_weights=(0.35, 0.35, 0.30, 0.35))
        return Workload("c1: 76+10+76 flexible linker, 32 replicas", [sim], table, V, S, seed=seed)
    if cid == 2:
        table = contact_table(rng, with_crowder=True, crowder_eps=0.1)
        lengths = list(rng.integers(60, 161, size=24))
        sim = rigid_sim(rng, lengths, 250.0, 32, sigma_type, crowders=40)
        return Workload("c2: 24 proteins U[60,160] + 40 crowders x20, box 250 A, 32 replicas", [sim], table,
                        seed=seed)
    if cid == 3:
        table = contact_table(rng)
        sims = []
        for _ in range(96):
            nm = int(rng.integers(2, 13))
            lengths = [int(round(math.exp(rng.uniform(math.log(40), math.log(400))))) for _ in range(nm)]
            nrep = int(rng.integers(8, 41))
            box = max(150.0, 2.2 * (sum(lengths) * 2000.0) ** (1 / 3))
            sims.append(rigid_sim(rng, lengths, box, nrep, sigma_type))
        return Workload("c3: 96 uneven simulations", sims, table, seed=seed)
    if cid == 4:
        table = contact_table(rng)
        base = compact_chain(rng, 76)
        t, q, s = residue_params(rng, 76, sigma_type)
        centres = place_centres(rng, [12.0] * 8, 120.0)
        mols = [Molecule(base + np.asarray(c, np.float32), t, q, s) for c in centres]
        sim = Simulation(mols, 120.0, ladder(288.0, 450.0, 32), ladder(0.5, 2.0, 32), ladder(0.2, 0.2, 32))
        return Workload("c4: 8x76 copies, box 120 A, 32 replicas", [sim], table, seed=seed)
    raise ValueError("unknown configuration %r" % (config,))
