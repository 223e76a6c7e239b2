"""Seeded synthetic ChIMES workloads.

Two things are generated here, both deterministic for a given seed:

* parameter files in the ChIMES text format, i.e. the exact layout that
  ``chimesFF::read_parameters`` parses (chimesFF/src/chimesFF.cpp:354-1570):
  ``PAIRTYP: CHEBYSHEV o2 o3 o4``, ``ATOM TYPES``, ``# TYPEIDX #`` rows,
  ``ATOM PAIRS`` with 8-column ``# PAIRIDX #`` rows (S_DELTA present, MORSE
  lambda last), ``FCUT TYPE``, ``SPECIAL 3B/4B S_MAXIM/S_MINIM``,
  ``PAIRTYPE PARAMS`` (exactly o2 ``pow coeff`` lines),
  ``TRIPLETTYPE PARAMS`` / ``QUADRUPLETYPE PARAMS`` blocks (powers in columns
  1..P, coefficient in column P+3), ``PAIRMAPS``/``TRIPMAPS``/``QUADMAPS`` whose
  keys concatenate the proper pair names in ij,ik,jk / ij,ik,il,jk,jl,kl order
  (chimesFF.cpp:976-1005, 1307-1349), and ``ENDFILE``;
* periodic configurations: positions by random sequential insertion with a
  minimum-image rejection radius, and element labels drawn at random.

Many-body power tuples are listed once per orbit of the label-preserving atom
permutations of the cluster type ("deduplicated"): TOTAL = UNIQUE = number of
orbit representatives.  ``expand=True`` instead lists every member of each
orbit with the orbit's shared coefficient, which is how the published ChIMES
files are laid out (e.g. ``UNIQUE: 30 TOTAL: 112``).

Powers run over [0, order-1]: the reference indexes ``Tn[pow]`` in vectors of
length order+1 (chimesFF.h:46, chimesFF.cpp:2081), so order-1 is the largest
power a 3B/4B term may use without reading past its polynomial table.
"""

from __future__ import annotations

import dataclasses
import itertools
import math
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

ELEMENTS = ("C", "N", "O")
MASSES = {"C": 12.011, "N": 14.0067, "O": 15.9994}


# ----------------------------------------------------------------------------
# Cluster-type combinatorics
# ----------------------------------------------------------------------------

def pair_slots(n_atoms: int) -> List[Tuple[int, int]]:
    """Pair order of a cluster: ij, ik, jk (3B) / ij, ik, il, jk, jl, kl (4B)."""
    return [(i, j) for i in range(n_atoms) for j in range(i + 1, n_atoms)]


def _label_group(atoms: Sequence[int]) -> List[Tuple[int, ...]]:
    n = len(atoms)
    return [s for s in itertools.permutations(range(n))
            if all(atoms[s[i]] == atoms[i] for i in range(n))]


def _pair_permutation(sigma: Sequence[int], n_atoms: int) -> List[int]:
    slots = pair_slots(n_atoms)
    index = {p: k for k, p in enumerate(slots)}
    out = []
    for (i, j) in slots:
        a, b = sigma[i], sigma[j]
        out.append(index[(min(a, b), max(a, b))])
    return out


def power_orbits(atoms: Sequence[int], order: int, min_nonzero: int) -> List[List[Tuple[int, ...]]]:
    """Orbits of power tuples in [0, order-1]^P with >= min_nonzero nonzero
    entries under the label-preserving permutations of the cluster's atoms.
    Each orbit is returned as a list whose first member is its lexicographically
    smallest tuple (the representative); orbits are ordered by representative."""
    n = len(atoms)
    npairs = n * (n - 1) // 2
    perms = [_pair_permutation(s, n) for s in _label_group(atoms)]
    seen = set()
    orbits = []
    for p in itertools.product(range(order), repeat=npairs):
        if sum(1 for v in p if v) < min_nonzero or p in seen:
            continue
        members = set()
        for perm in perms:
            q = [0] * npairs
            for k in range(npairs):
                q[perm[k]] = p[k]
            members.add(tuple(q))
        seen |= members
        orbits.append(sorted(members))
    return orbits


# ----------------------------------------------------------------------------
# Parameter files
# ----------------------------------------------------------------------------

@dataclasses.dataclass
class ParamSpec:
    """Recipe for one synthetic parameter set.

    ``rin``/``rout``/``lam`` are either one value for every pair type or a
    (low, high) range sampled per pair type.  ``s3max`` etc. are ``None``
    (keep the 2B-derived defaults), a float (``ALL v``) or a dict mapping a
    triplet/quadruplet type index to per-pair values (``SPECIFIC``)."""
    elements: Sequence[str]
    orders: Tuple[int, int, int] = (12, 8, 0)
    rin: object = 1.0
    rout: object = 5.0
    lam: object = 1.4
    fcut: Tuple = ("TERSOFF", 0.5)
    s3max: object = None
    s3min: object = None
    s4max: object = None
    s4min: object = None
    excluded3: Tuple[int, ...] = ()
    excluded4: Tuple[int, ...] = ()
    energy_offsets: Optional[Sequence[float]] = None
    penalty: Optional[Tuple[float, float]] = None
    coeff_sigma: float = 0.05
    expand: bool = False
    seed: int = 1000


def _draw(v, rng):
    if isinstance(v, (tuple, list)):
        return float(rng.uniform(v[0], v[1]))
    return float(v)


def _fmt(x: float) -> str:
    return repr(float(x))


def build_param_text(spec: ParamSpec) -> str:
    rng = np.random.default_rng(spec.seed)
    el = list(spec.elements)
    nt = len(el)
    o2, o3, o4 = spec.orders
    pairs = [(a, b) for a in range(nt) for b in range(a, nt)]
    pidx = {p: k for k, p in enumerate(pairs)}

    def proper(a, b):
        a, b = min(a, b), max(a, b)
        return el[a] + el[b]

    pair_rin = [_draw(spec.rin, rng) for _ in pairs]
    pair_rout = [_draw(spec.rout, rng) for _ in pairs]
    pair_lam = [_draw(spec.lam, rng) for _ in pairs]

    L = []
    w = L.append
    w("! Synthetic ChIMES parameter set (seeded generator)")
    w("! seed = %d" % spec.seed)
    w("")
    w("PAIRTYP: CHEBYSHEV  %d %d %d -1 1" % (o2, o3, o4))
    w("")
    w("ATOM TYPES: %d" % nt)
    w("")
    w("# TYPEIDX #\t# ATM_TYP #\t# ATMCHRG #\t# ATMMASS #")
    for i, e in enumerate(el):
        w("%d\t\t%s\t\t0\t\t%s" % (i, e, MASSES.get(e, 10.0)))
    w("")
    w("ATOM PAIRS: %d" % len(pairs))
    w("")
    w("# PAIRIDX #\t# ATM_TY1 #\t# ATM_TY1 #\t# S_MINIM #\t# S_MAXIM #\t# S_DELTA #\t# CHBDIST #\t# MORSE_LAMBDA #")
    for k, (a, b) in enumerate(pairs):
        w("\t%d\t%s\t%s\t%s\t%s\t0.01\tMORSE\t%s" % (k, el[a], el[b], _fmt(pair_rin[k]),
                                                      _fmt(pair_rout[k]), _fmt(pair_lam[k])))
    w("")
    if spec.penalty is not None:
        w("PAIR CHEBYSHEV PENALTY DIST: %s" % _fmt(spec.penalty[0]))
        w("PAIR CHEBYSHEV PENALTY SCALING: %s" % _fmt(spec.penalty[1]))
        w("")
    if spec.fcut[0] == "TERSOFF":
        w("FCUT TYPE: TERSOFF %s" % _fmt(spec.fcut[1]))
    else:
        w("FCUT TYPE: CUBIC")
    w("")

    trips = list(itertools.combinations_with_replacement(range(nt), 3)) if o3 > 0 else []
    quads = list(itertools.combinations_with_replacement(range(nt), 4)) if o4 > 0 else []
    trip_pairs = [[proper(t[i], t[j]) for (i, j) in pair_slots(3)] for t in trips]
    quad_pairs = [[proper(q[i], q[j]) for (i, j) in pair_slots(4)] for q in quads]

    def special(tag, val, types, tpairs, maps_key):
        if val is None:
            return
        if isinstance(val, dict):
            w("%s SPECIFIC %d" % (tag, len(val)))
            for t, cuts in sorted(val.items()):
                w("%s %s %s" % (maps_key[t], " ".join(tpairs[t]), " ".join(_fmt(c) for c in cuts)))
        else:
            w("%s ALL %s" % (tag, _fmt(val)))
        w("")

    # SPECIFIC rows are looked up by a map key; use the key of the type's own
    # (sorted) atom order.
    trip_key = {ti: "".join(trip_pairs[ti]) for ti in range(len(trips))}
    quad_key = {qi: "".join(quad_pairs[qi]) for qi in range(len(quads))}

    if o3 > 0:
        special("SPECIAL 3B S_MAXIM:", spec.s3max, trips, trip_pairs, trip_key)
        special("SPECIAL 3B S_MINIM:", spec.s3min, trips, trip_pairs, trip_key)
    if o4 > 0:
        special("SPECIAL 4B S_MAXIM:", spec.s4max, quads, quad_pairs, quad_key)
        special("SPECIAL 4B S_MINIM:", spec.s4min, quads, quad_pairs, quad_key)

    if o3 > 0:
        w("ATOM PAIR TRIPLETS: %d" % len(trips))
    if o4 > 0:
        w("ATOM PAIR QUADRUPLETS: %d" % len(quads))
    w("")
    w("PAIR CHEBYSHEV PARAMS ")
    w("")
    for k, (a, b) in enumerate(pairs):
        w("PAIRTYPE PARAMS: %d %s %s" % (k, el[a], el[b]))
        w("")
        for pw in range(o2):
            c = rng.normal(0.0, spec.coeff_sigma) / (1.0 + pw)
            w("%d %s" % (pw, _fmt(c)))
        w(" ")

    def cluster_block(title, head, idx, atoms, pnames, order, min_nz, excluded):
        w(title)
        w("   INDEX: %d ATOMS: %s" % (idx, " ".join(el[a] for a in atoms)))
        if idx in excluded:
            w("PAIRS: %s EXCLUDED: 0 TOTAL: 0" % " ".join(pnames))
            w("")
            return
        orbits = power_orbits(atoms, order, min_nz)
        rows = []
        for oi, orb in enumerate(orbits):
            c = rng.normal(0.0, spec.coeff_sigma) / (1.0 + sum(orb[0]))
            members = orb if spec.expand else orb[:1]
            for m in members:
                rows.append((m, oi, c))
        w("PAIRS: %s UNIQUE: %d TOTAL: %d" % (" ".join(pnames), len(orbits), len(rows)))
        w(head)
        w("   " + "-" * 76)
        for r, (m, oi, c) in enumerate(rows):
            w("%d %s %d %d %s" % (r, " ".join(str(v) for v in m), oi, oi, _fmt(c)))
        w("")

    if o3 > 0:
        w("TRIPLET CHEBYSHEV PARAMS ")
        w("")
        for ti, t in enumerate(trips):
            cluster_block("TRIPLETTYPE PARAMS:",
                          "     index  |  powers  |  equiv index  |  param index  |       parameter       ",
                          ti, t, trip_pairs[ti], o3, 2, set(spec.excluded3))
    if o4 > 0:
        w("QUADRUPLET CHEBYSHEV PARAMS ")
        w("")
        for qi, q in enumerate(quads):
            cluster_block("QUADRUPLETYPE PARAMS: ",
                          "     index  |  powers  |  equiv index  |  param index  |       parameter       ",
                          qi, q, quad_pairs[qi], o4, 3, set(spec.excluded4))

    pmap = {}
    for a in range(nt):
        for b in range(nt):
            pmap[el[a] + el[b]] = pidx[(min(a, b), max(a, b))]
    w("")
    w("PAIRMAPS: %d" % len(pmap))
    for k in sorted(pmap):
        w("%d %s" % (pmap[k], k))
    w("")
    if o3 > 0:
        tmap = {}
        for t in itertools.product(range(nt), repeat=3):
            key = proper(t[0], t[1]) + proper(t[0], t[2]) + proper(t[1], t[2])
            ti = trips.index(tuple(sorted(t)))
            tmap[key] = -1 if ti in spec.excluded3 else ti
        w("TRIPMAPS: %d" % len(tmap))
        for k in sorted(tmap):
            w("%d %s" % (tmap[k], k))
        w("")
    if o4 > 0:
        qmap = {}
        for q in itertools.product(range(nt), repeat=4):
            key = "".join(proper(q[i], q[j]) for (i, j) in pair_slots(4))
            qi = quads.index(tuple(sorted(q)))
            qmap[key] = -1 if qi in spec.excluded4 else qi
        w("QUADMAPS: %d" % len(qmap))
        for k in sorted(qmap):
            w("%d %s" % (qmap[k], k))
        w("")
    if spec.energy_offsets is not None:
        w("NO ENERGY OFFSETS: %d" % nt)
        for i in range(nt):
            w("ENERGY OFFSET %d %s" % (i + 1, _fmt(spec.energy_offsets[i])))
    w("ENDFILE")
    return "\n".join(L) + "\n"


def write_param_file(path: str, spec: ParamSpec) -> str:
    with open(path, "w") as f:
        f.write(build_param_text(spec))
    return path


# ----------------------------------------------------------------------------
# Configurations
# ----------------------------------------------------------------------------

@dataclasses.dataclass
class Config:
    types: List[str]
    pos: np.ndarray          # (N, 3) Cartesian, Angstrom
    cell: np.ndarray         # (3, 3) rows are the a, b, c lattice vectors

    @property
    def n_atoms(self) -> int:
        return len(self.types)

    def xyz_text(self) -> str:
        c = self.cell.reshape(-1)
        out = ["%d" % self.n_atoms, " ".join(_fmt(v) for v in c)]
        for t, p in zip(self.types, self.pos):
            out.append("%s %s %s %s" % (t, _fmt(p[0]), _fmt(p[1]), _fmt(p[2])))
        return "\n".join(out) + "\n"

    def write_xyz(self, path: str) -> str:
        with open(path, "w") as f:
            f.write(self.xyz_text())
        return path


def read_xyz(path: str) -> Config:
    """Reads the .xyz layout of the reference's example drivers: atom count,
    a comment line holding the 9 cell-vector components, then ``type x y z``."""
    with open(path) as f:
        lines = f.read().splitlines()
    n = int(lines[0].split()[0])
    cell = np.array([float(v) for v in lines[1].split()[:9]]).reshape(3, 3)
    types, pos = [], []
    for ln in lines[2:2 + n]:
        w = ln.split()
        types.append(w[0])
        pos.append([float(w[1]), float(w[2]), float(w[3])])
    return Config(types, np.array(pos, dtype=np.float64), cell)


def random_config(n_atoms: int, cell, elements: Sequence[str], rmin: float, seed: int,
                  type_probs: Optional[Sequence[float]] = None, max_tries: int = 200000) -> Config:
    """Random sequential insertion: uniform fractional coordinates, rejected when
    the minimum-image distance to any accepted atom is below ``rmin``."""
    rng = np.random.default_rng(seed)
    cell = np.asarray(cell, dtype=np.float64).reshape(3, 3)
    ortho = np.allclose(cell - np.diag(np.diag(cell)), 0.0)
    frac = np.zeros((n_atoms, 3))
    n = 0
    tries = 0
    if ortho and n_atoms > 1500:
        lengths = np.diag(cell)
        ncell = np.maximum((lengths // rmin).astype(int), 1)
        grid: Dict[Tuple[int, int, int], List[int]] = {}
        while n < n_atoms:
            tries += 1
            if tries > max_tries * 10:
                raise RuntimeError("random_config: packing too dense")
            f = rng.random(3)
            c = tuple((f * ncell).astype(int) % ncell)
            cand = []
            for d in itertools.product((-1, 0, 1), repeat=3):
                cand.extend(grid.get(tuple((np.array(c) + d) % ncell), ()))
            if cand:
                df = frac[cand] - f
                df -= np.round(df)
                r = np.sqrt(((df * lengths) ** 2).sum(axis=1))
                if r.min() < rmin:
                    continue
            frac[n] = f
            grid.setdefault(c, []).append(n)
            n += 1
    else:
        while n < n_atoms:
            tries += 1
            if tries > max_tries:
                raise RuntimeError("random_config: packing too dense")
            f = rng.random(3)
            if n:
                df = frac[:n] - f
                df -= np.round(df)
                r = np.sqrt(((df @ cell) ** 2).sum(axis=1))
                if r.min() < rmin:
                    continue
            frac[n] = f
            n += 1
    pos = frac @ cell
    probs = None if type_probs is None else np.asarray(type_probs, dtype=np.float64)
    tidx = rng.choice(len(elements), size=n_atoms, p=probs)
    return Config([elements[i] for i in tidx], pos, cell)


def random_config_batched(n_atoms: int, cell, elements: Sequence[str], rmin: float, seed: int,
                          batch: Optional[int] = None, max_rounds: int = 100000) -> Config:
    """Random insertion with rejection, vectorised: candidates (uniform
    fractional coordinates) are drawn ``batch`` at a time; a candidate is kept
    when its minimum-image distance to every accepted atom and to every earlier
    candidate of its batch is at least ``rmin``.  Every pair of the result is
    at least ``rmin`` apart, as with ``random_config``; the random stream
    differs.  Used for the many few-thousand-atom configurations of the
    batched and serving workloads, where the one-candidate-at-a-time loop
    dominates the set-up time.  The default batch, sqrt(2 V / v) with v the
    volume of an ``rmin`` sphere, keeps conflicts inside a batch to about
    one."""
    rng = np.random.default_rng(seed)
    cell = np.asarray(cell, dtype=np.float64).reshape(3, 3)
    if batch is None:
        vol = abs(float(np.linalg.det(cell)))
        batch = int(min(256, max(4, math.sqrt(2.0 * vol / (4.18879 * rmin ** 3)))))
    frac = np.zeros((n_atoms, 3))
    n = 0
    r2 = rmin * rmin
    # orthorhombic cells of at least three rmin-sized bins per axis: accepted
    # atoms are kept in a bin grid (up to K per bin) and a candidate is tested
    # against the 27 bins around its own; otherwise against every accepted atom
    lengths = np.diag(cell)
    ortho = np.allclose(cell - np.diag(lengths), 0.0)
    m = (lengths // rmin).astype(int) if ortho else np.zeros(3, dtype=int)
    use_grid = ortho and bool(np.all(m >= 3))
    K = 4
    if use_grid:
        grid = np.full((m[0], m[1], m[2], K, 3), 10.0)       # empty slots sit far outside the cell
        fill = np.zeros((m[0], m[1], m[2]), dtype=int)
        offs = np.array([[a, b, c] for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)])
    for _ in range(max_rounds):
        if n >= n_atoms:
            break
        cand = rng.random((batch, 3))
        ok = np.ones(batch, dtype=bool)
        if use_grid and n:
            cb = (cand * m).astype(int) % m
            nb = (cb[:, None, :] + offs[None, :, :]) % m                       # (B, 27, 3)
            other = grid[nb[..., 0], nb[..., 1], nb[..., 2]]                   # (B, 27, K, 3)
            df = other - cand[:, None, None, :]
            df -= np.round(df)
            ok &= (((df * lengths) ** 2).sum(axis=3) >= r2).all(axis=(1, 2))
        elif n:
            for a in range(0, n, 2048):
                df = cand[:, None, :] - frac[None, a:min(n, a + 2048), :]
                df -= np.round(df)
                ok &= (np.einsum("ijk,kl->ijl", df, cell) ** 2).sum(axis=2).min(axis=1) >= r2
        df = cand[:, None, :] - cand[None, :, :]
        df -= np.round(df)
        close = np.triu((np.einsum("ijk,kl->ijl", df, cell) ** 2).sum(axis=2) < r2, k=1)
        ok &= ~close.any(axis=0)           # no earlier candidate of the batch within rmin
        c = cand[ok][:n_atoms - n]
        if use_grid and len(c):
            cb = (c * m).astype(int) % m
            lin = (cb[:, 0] * m[1] + cb[:, 1]) * m[2] + cb[:, 2]
            order = np.argsort(lin, kind="stable")
            lin, c = lin[order], c[order]
            first = np.r_[True, lin[1:] != lin[:-1]]
            rank = np.arange(len(lin)) - np.maximum.accumulate(np.where(first, np.arange(len(lin)), 0))
            slot = fill.reshape(-1)[lin] + rank
            keep = slot < K                # a full bin drops the candidate (never at these densities)
            lin, slot, c = lin[keep], slot[keep], c[keep]
            grid.reshape(-1, K, 3)[lin, slot] = c
            np.add.at(fill.reshape(-1), lin, 1)
        frac[n:n + len(c)] = c
        n += len(c)
    if n < n_atoms:
        raise RuntimeError("random_config_batched: packing too dense")
    pos = frac @ cell
    tidx = rng.choice(len(elements), size=n_atoms)
    return Config([elements[i] for i in tidx], pos, cell)


# ----------------------------------------------------------------------------
# The named workloads (seed = 1000 + workload number)
# ----------------------------------------------------------------------------

def spec_c1() -> ParamSpec:
    """1 element; 2B order 12 (rin 1.0, rout 5.0, lambda 1.4); 3B order 8 with
    outer cutoff 4.0; Tersoff cutoff with offset 0.5; no 4B."""
    return ParamSpec(elements=["C"], orders=(12, 8, 0), rin=1.0, rout=5.0, lam=1.4,
                     fcut=("TERSOFF", 0.5), s3max=4.0, seed=1001)


def config_c1() -> Config:
    return random_config(64, np.diag([9.0, 9.0, 9.0]), ["C"], 1.2, seed=1101)


def spec_c2(elements=("C", "N"), orders=(12, 8, 4), seed=1002) -> ParamSpec:
    """Per pair type: 2B order 12, rin 0.9, rout 5.0, lambda ~ U(1.3, 1.6);
    3B order 8 with outer 4.0; 4B order 4 with outer 3.2."""
    return ParamSpec(elements=list(elements), orders=orders, rin=0.9, rout=5.0, lam=(1.3, 1.6),
                     fcut=("TERSOFF", 0.5), s3max=4.0, s4max=3.2, seed=seed)


def config_c2(n_atoms=1024, box=22.0, seed=1102) -> Config:
    return random_config(n_atoms, np.diag([box, box, box]), ["C", "N"], 1.0, seed=seed,
                         type_probs=[0.5, 0.5])


def spec_c3() -> ParamSpec:
    return spec_c2(orders=(12, 10, 4), seed=1003)


def config_c3(n_atoms=32768, box=(70.0, 70.0, 72.0), seed=1103) -> Config:
    return random_config(n_atoms, np.diag(box), ["C", "N"], 1.0, seed=seed, type_probs=[0.5, 0.5])


def spec_c4() -> ParamSpec:
    """Three-element parameter set of the 12/10/4 recipe; each batched
    configuration uses one, two or all three of its elements."""
    return spec_c2(elements=("C", "N", "O"), orders=(12, 10, 4), seed=1004)


def _gen_config(args):
    n, L, elements, seed = args
    return random_config_batched(n, np.diag([L, L, L]), elements, 1.0, seed=seed)


def generate_configs(jobs, processes: int = 0) -> List[Config]:
    """Configurations for (n_atoms, box side, elements, seed) jobs, in a pool
    of ``processes`` spawned workers when that is above 1 (each job has its
    own seed, so the result does not depend on the pool)."""
    if processes and processes > 1 and len(jobs) > 64:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(processes) as pool:
            return pool.map(_gen_config, jobs, chunksize=max(1, len(jobs) // (8 * processes)))
    return [_gen_config(j) for j in jobs]


def configs_c4(n_configs=4096, seed=1104, n_min=8, n_max=512, processes: int = 0) -> List[Config]:
    """Atom counts log-uniform in [n_min, n_max], densities U(0.05, 0.12) per
    cubic Angstrom, 1-3 elements per configuration."""
    rng = np.random.default_rng(seed)
    jobs = []
    for c in range(n_configs):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        rho = rng.uniform(0.05, 0.12)
        L = (n / rho) ** (1.0 / 3.0)
        ne = int(rng.integers(1, 4))
        jobs.append((n, L, list(ELEMENTS[:ne]), int(rng.integers(1 << 31))))
    return generate_configs(jobs, processes)


def specs_c5() -> List[ParamSpec]:
    """Three parameter sets for the serving workload: 12/8/4 with one element,
    12/10/4 with two, 12/8/4 with three."""
    return [spec_c2(elements=("C",), orders=(12, 8, 4), seed=1051),
            spec_c2(elements=("C", "N"), orders=(12, 10, 4), seed=1052),
            spec_c2(elements=("C", "N", "O"), orders=(12, 8, 4), seed=1053)]


# ----------------------------------------------------------------------------
# Tabulated parameter sets (the reference's TABULATION option)
# ----------------------------------------------------------------------------
def _tab_g(r, rc, lam):
    """Smooth decaying radial factor exp(-r/lam) (1 - r/rc)^3 and its derivative (0 past rc)."""
    r = np.asarray(r, dtype=np.float64)
    inside = r < rc
    u = np.where(inside, 1.0 - r / rc, 0.0)
    ex = np.exp(-r / lam)
    g = ex * u ** 3
    dg = -ex / lam * u ** 3 - 3.0 * ex * u ** 2 / rc
    return g, np.where(inside, dg, 0.0)


def _write_rows(path: str, rows: np.ndarray) -> None:
    with open(path, "w") as f:
        f.write("%d\n" % len(rows))
        f.write("\n".join(" ".join(repr(float(v)) for v in row) for row in rows))
        f.write("\n")


def write_tabulated_param_file(path: str, spec: ParamSpec, tab2: bool = True, tab3: bool = True,
                               r0_2: float = 0.5, step2: float = 0.005, r0_3: float = 0.8,
                               step3: float = 0.1, seed: int = 7) -> str:
    """Writes ``spec``'s parameter file with its 2-body and/or 3-body terms
    tabulated, as the reference's TABULATION build reads them
    (chimesFF.cpp:199-351, 719-769, 882-934): ``PAIRTYPE PARAMS: k A B TABULATED
    <name>`` and ``INDEX: t ATOMS: a b c TABULATED <name>`` lines (the
    coefficient rows stay and are ignored), and beside the file, for each
    table, ``<name>.energy`` and ``<name>.force``.

    The tabulated energies are seeded smooth functions, not a Chebyshev fit:
    2-body E(r) = A_k g(r), 3-body E = B_t g(r_ij) g(r_ik) g(r_jk) with
    g(r) = exp(-r/1.4) (1 - r/rc)^3, and the force columns are (dE/dr_p)/r_p,
    the scalar that multiplies the pair vector r_j - r_i in compute_2B_tab /
    compute_3B_tab.  2-body grids run from ``r0_2`` in steps of ``step2`` to
    past the pair's outer cutoff; 3-body grids are n x n x n points from
    ``r0_3`` in steps of ``step3`` (rij slowest, rjk fastest) covering the
    largest 3-body cutoff."""
    import os
    text = build_param_text(spec)
    rng = np.random.default_rng(seed)
    base = os.path.splitext(os.path.basename(path))[0]
    out_dir = os.path.dirname(os.path.abspath(path))
    lines = text.split("\n")
    # pair cutoffs and the largest 3-body outer cutoff, from the file itself
    rout = {}
    in_pairs = False
    s3_all = None
    for ln in lines:
        t = ln.split()
        if ln.startswith("# PAIRIDX #"):
            in_pairs = True
            continue
        if in_pairs:
            if len(t) == 8:
                rout[int(t[0])] = float(t[4])
                continue
            in_pairs = False
        if ln.startswith("SPECIAL 3B S_MAXIM: ALL"):
            s3_all = float(t[4])
    rc3 = s3_all if s3_all is not None else max(rout.values())
    if isinstance(spec.s3max, dict):
        rc3 = max([rc3] + [max(v) for v in spec.s3max.values()])
    out = []
    after_trip_header = False
    for ln in lines:
        t = ln.split()
        if tab2 and ln.startswith("PAIRTYPE PARAMS:"):
            k = int(t[2])
            name = "%s_2b.type_%d.dat" % (base, k)
            n = int(math.ceil((rout[k] + 2 * step2 - r0_2) / step2)) + 1
            r = r0_2 + step2 * np.arange(n)
            g, dg = _tab_g(r, rout[k], 1.4)
            amp = float(rng.uniform(5.0, 20.0))
            _write_rows(os.path.join(out_dir, name + ".energy"), np.stack([r, amp * g], axis=1))
            _write_rows(os.path.join(out_dir, name + ".force"), np.stack([r, amp * dg / r], axis=1))
            ln = ln + " TABULATED " + name
        if tab3 and after_trip_header and ln.strip().startswith("INDEX:"):
            ti = int(t[1])
            name = "%s_3b.type_%d.dat" % (base, ti)
            n = int(math.ceil((rc3 + 2 * step3 - r0_3) / step3)) + 1
            ax = r0_3 + step3 * np.arange(n)
            rij, rik, rjk = (a.ravel() for a in np.meshgrid(ax, ax, ax, indexing="ij"))
            gij, dij = _tab_g(rij, rc3, 1.4)
            gik, dik = _tab_g(rik, rc3, 1.4)
            gjk, djk = _tab_g(rjk, rc3, 1.4)
            amp = float(rng.uniform(1.0, 4.0))
            e = amp * gij * gik * gjk
            fij = amp * dij * gik * gjk / rij
            fik = amp * gij * dik * gjk / rik
            fjk = amp * gij * gik * djk / rjk
            _write_rows(os.path.join(out_dir, name + ".energy"), np.stack([rij, rik, rjk, e], axis=1))
            _write_rows(os.path.join(out_dir, name + ".force"), np.stack([rij, rik, rjk, fij, fik, fjk], axis=1))
            ln = ln + " TABULATED " + name
        after_trip_header = ln.startswith("TRIPLETTYPE PARAMS:")
        out.append(ln)
    with open(path, "w") as f:
        f.write("\n".join(out))
    return path


# ----------------------------------------------------------------------------
# LAMMPS-style inputs: local atoms, ghost images and full neighbour lists
# ----------------------------------------------------------------------------
@dataclasses.dataclass
class NeighborData:
    """What a LAMMPS pair style sees on one rank: nall = local + ghost atoms
    (positions x, ChIMES type indices, global tags; ghosts carry their owner's
    tag), and full neighbour lists of the local atoms (ilist order), with
    neighbours concatenated in `neigh`."""
    x: np.ndarray            # (nall, 3)
    type: np.ndarray         # (nall,) int32
    tag: np.ndarray          # (nall,) int64
    nlocal: int
    ilist: np.ndarray        # (inum,) int32
    numneigh: np.ndarray     # (inum,) int32
    neigh: np.ndarray        # (sum numneigh,) int32
    owner: np.ndarray        # (nall,) local atom each atom images


def lammps_neighbors(cfg: Config, type_idx: np.ndarray, cutoff: float, seed: Optional[int] = None) -> NeighborData:
    """Ghost atoms: every periodic image of a local atom within `cutoff` of the
    cell (fractional margin cutoff / perpendicular height on each axis), as
    LAMMPS's communication builds them; neighbour lists: every other atom
    (local or ghost) within `cutoff` of each local atom.  `seed` shuffles each
    list (LAMMPS lists come in bin order, not sorted)."""
    cell = np.asarray(cfg.cell, dtype=np.float64)
    inv = np.linalg.inv(cell)
    frac = cfg.pos @ inv
    frac -= np.floor(frac)
    n = cfg.n_atoms
    vol = abs(np.linalg.det(cell))
    heights = [vol / np.linalg.norm(np.cross(cell[(k + 1) % 3], cell[(k + 2) % 3])) for k in range(3)]
    margin = np.array([cutoff / h for h in heights])
    reach = [int(math.ceil(m)) for m in margin]
    xs, owners = [frac @ cell], [np.arange(n)]
    for sa in range(-reach[0], reach[0] + 1):
        for sb in range(-reach[1], reach[1] + 1):
            for sc in range(-reach[2], reach[2] + 1):
                if sa == 0 and sb == 0 and sc == 0:
                    continue
                fs = frac + np.array([sa, sb, sc], dtype=np.float64)
                keep = np.all((fs >= -margin) & (fs < 1.0 + margin), axis=1)
                if keep.any():
                    xs.append(fs[keep] @ cell)
                    owners.append(np.nonzero(keep)[0])
    x = np.concatenate(xs)
    owner = np.concatenate(owners)
    rng = np.random.default_rng(seed) if seed is not None else None
    numneigh, neigh = [], []
    for i in range(n):
        d = np.linalg.norm(x - x[i], axis=1)
        nb = np.nonzero(d < cutoff)[0]
        nb = nb[nb != i]
        if rng is not None:
            nb = rng.permutation(nb)
        numneigh.append(len(nb))
        neigh.append(nb)
    return NeighborData(x=np.ascontiguousarray(x), type=np.ascontiguousarray(np.asarray(type_idx)[owner], dtype=np.int32),
                        tag=(owner + 1).astype(np.int64), nlocal=n, ilist=np.arange(n, dtype=np.int32),
                        numneigh=np.array(numneigh, dtype=np.int32),
                        neigh=np.ascontiguousarray(np.concatenate(neigh).astype(np.int32)), owner=owner)
