"""Seeded synthetic workloads for the structure-factor path.

No public dataset is involved: every input is drawn from a numpy PCG64
generator with a fixed seed, with the shapes and value distributions of the
five benchmark configurations

* ``config0``: 32 atoms (12 C, 12 H, 4 N, 4 O), P2_1/c, sin(theta)/lambda <= 0.8,
  anisotropic non-H atoms, multipoles to l = 4, one type per atom;
* ``config1``: 5,000 atoms in protein ratios, P2_1 2_1 2_1, 60x70x80 A,
  d >= 1.5 A, isotropic B ~ U(10,40), 150 shared types;
* ``config2``: 50,000 atoms, P4_3 2_1 2, 120x120x140 A, d >= 1.2 A,
  anisotropic non-H, 300 types, full derivative set;
* ``config4``: a batch of crystals with tabulated form factors
  (``config4_specs`` / ``config4_crystal`` / ``config4_f0``);

and small cases used by the tests.  Synthetic wavefunctions: every element
gets a core and a valence orbital of two Slater functions each (hydrogen: a
valence orbital only), normalised to one, so f_core(0) and f_val(0) count
electrons the way Clementi-Roetti wavefunctions do in the reference.
"""
from __future__ import annotations

import math

import numpy as np

from .crystal import space_group, unique_hkl, convert_adp, frac_to_cart_matrix
from .model import AtomType, Orbital, Structure, Wavefunction

BOHR = 0.529177  # Angstrom

_ELEMENTS = {
    #      Z  core occ, valence occ, core exps (1/bohr), valence exps, core pow, val pow, anomalous
    "H": (1, 0, 1, (), (1.0, 1.6), (), (0, 0), 0j),
    "C": (6, 2, 4, (5.4, 8.0), (1.6, 2.6), (0, 0), (1, 1), 0.0033 + 0.0016j),
    "N": (7, 2, 5, (6.4, 9.4), (1.9, 3.0), (0, 0), (1, 1), 0.0061 + 0.0033j),
    "O": (8, 2, 6, (7.4, 10.8), (2.2, 3.4), (0, 0), (1, 1), 0.0106 + 0.0060j),
    "S": (16, 10, 6, (14.0, 6.0), (1.8, 2.9), (0, 1), (2, 2), 0.1246 + 0.1234j),
}
_DEF_POW = {"H": [0, 1, 2], "C": [2, 2, 2, 3, 4], "N": [2, 2, 2, 3, 4],
            "O": [2, 2, 2, 3, 4], "S": [4, 4, 4, 4, 4]}


def _norm_orbital(powers, exps, coeffs):
    """scale coefficients so that int R(r)^2 r^2 dr = 1."""
    s = 0.0
    for p, a, c in zip(powers, exps, coeffs):
        for q, b, d in zip(powers, exps, coeffs):
            n = p + q + 2
            s += c * d * math.factorial(n) / (a + b) ** (n + 1)
    f = 1.0 / math.sqrt(s)
    return [c * f for c in coeffs]


def make_wavefunction(symbol, rng):
    z, occ_core, occ_val, ce, ve, cp, vp, anom = _ELEMENTS[symbol]
    orbitals, occ, core, val = [], [], [], []
    if ce:
        exps = [e / BOHR * rng.uniform(0.95, 1.05) for e in ce]
        coeffs = _norm_orbital(cp, exps, [1.0, rng.uniform(0.2, 0.6)])
        orbitals.append(Orbital(list(cp), exps, coeffs))
        occ.append(occ_core)
        core.append(len(orbitals) - 1)
    exps = [e / BOHR * rng.uniform(0.95, 1.05) for e in ve]
    coeffs = _norm_orbital(vp, exps, [1.0, rng.uniform(0.2, 0.6)])
    orbitals.append(Orbital(list(vp), exps, coeffs))
    occ.append(occ_val)
    val.append(len(orbitals) - 1)
    zeta = rng.uniform(3.0, 5.0) / BOHR
    return Wavefunction(symbol, z, orbitals, occ, core, val, zeta, list(_DEF_POW[symbol]), anom)


def make_type(symbol, rng, l_max=4):
    if symbol == "H":
        l_max = min(l_max, 2)
    n_l = l_max + 1
    plm = np.zeros(25)
    plm[: n_l * n_l] = rng.normal(0.0, 0.05, n_l * n_l)
    return AtomType(plm, n_l, rng.uniform(3.0, 6.0), rng.uniform(0.9, 1.1), rng.uniform(0.9, 1.1))


def random_rotation(rng, allow_improper=False):
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    if allow_improper and rng.uniform() < 0.3:
        q[:, 2] = -q[:, 2]
    return q


def random_cell(rng, kind):
    if kind == "monoclinic":
        a, b, c = rng.uniform(8, 15, 3)
        return (a, b, c, 90.0, rng.uniform(95, 110), 90.0)
    if kind == "triclinic":
        a, b, c = rng.uniform(6, 12, 3)
        return (a, b, c, rng.uniform(80, 100), rng.uniform(95, 110), rng.uniform(80, 100))
    if kind == "hexagonal":
        a, c = rng.uniform(8, 15, 2)
        return (a, a, c, 90.0, 90.0, 120.0)
    a, b, c = rng.uniform(8, 15, 3)
    return (a, b, c, 90.0, 90.0, 90.0)


def jittered_positions(cell, n, rng, min_dist=1.0):
    """n fractional positions on a jittered grid: every pair of grid points
    is at least ``min_dist`` apart in Cartesian space."""
    m = frac_to_cart_matrix(cell)
    lengths = np.linalg.norm(m, axis=0)
    vol = abs(np.linalg.det(m))
    # grid spacing s (Angstrom) with n cells; jitter keeps min distance
    s = (vol / (n * 1.3)) ** (1.0 / 3.0)
    g = np.maximum(1, np.floor(lengths / s).astype(int))
    while np.prod(g) < n:
        g += 1
    cells = rng.choice(np.prod(g), size=n, replace=False)
    idx = np.stack(np.unravel_index(cells, tuple(g)), axis=1).astype(np.float64)
    step = 1.0 / g
    # the closest Cartesian approach of two grid cells, conservative
    spacing = np.min(lengths * step) * 0.5
    jit = max(0.0, (spacing - min_dist) / 2.0) / lengths
    frac = (idx + 0.5) * step + rng.uniform(-1, 1, (n, 3)) * np.minimum(jit, 0.45 * step)
    return frac % 1.0


def random_u_cart(rng, lo=0.01, hi=0.05):
    q = random_rotation(rng)
    ev = rng.uniform(lo, hi, 3)
    u = q @ np.diag(ev) @ q.T
    return np.array([u[0, 0], u[1, 1], u[2, 2], u[0, 1], u[0, 2], u[1, 2]])


def build_structure(*, cell, sg_symbol, elements, rng, n_types=None, hkl=None, stol_max=None,
                    d_min=None, aniso=True, iso_b=None, l_max=4, occupancy=(1.0, 1.0),
                    improper_lcs=False, anomalous_per_atom=False, name=""):
    """Assemble a Structure. ``elements`` is a list of element symbols, one
    per atom; with ``n_types`` None every atom gets its own type, otherwise
    atoms share ``n_types`` types (each used at least once, one element per
    type)."""
    sg = space_group(sg_symbol)
    n = len(elements)
    symbols = sorted(set(elements))
    wfns = [make_wavefunction(s, rng) for s in symbols]
    wfn_of = {s: i for i, s in enumerate(symbols)}
    atom_wfn = np.array([wfn_of[e] for e in elements], dtype=np.int32)
    types, atom_type = [], np.zeros(n, dtype=np.int32)
    if n_types is None:
        for i, e in enumerate(elements):
            types.append(make_type(e, rng, l_max))
            atom_type[i] = i
    else:
        # split the type budget among elements in proportion to their counts
        counts = {s: elements.count(s) for s in symbols}
        alloc = {s: max(1, int(round(n_types * counts[s] / n))) for s in symbols}
        while sum(alloc.values()) > n_types:
            s = max(alloc, key=lambda k: alloc[k])
            alloc[s] -= 1
        while sum(alloc.values()) < n_types:
            s = max(alloc, key=lambda k: counts[k] / alloc[k])
            alloc[s] += 1
        base = {}
        for s in symbols:
            base[s] = len(types)
            for _ in range(min(alloc[s], counts[s])):
                types.append(make_type(s, rng, l_max))
        seen = {s: 0 for s in symbols}
        for i, e in enumerate(elements):
            k = min(alloc[e], counts[e])
            j = seen[e]
            seen[e] += 1
            t = j if j < k else int(rng.integers(k))
            atom_type[i] = base[e] + t
    xyz = jittered_positions(cell, n, rng)
    adp = []
    for e in elements:
        if iso_b is not None:
            adp.append([rng.uniform(*iso_b) / (8 * math.pi ** 2)])
        elif aniso and e != "H":
            adp.append(list(convert_adp(cell, random_u_cart(rng), "U_cart", "U_cif")))
        else:
            adp.append([rng.uniform(0.02, 0.06)])
    occ = rng.uniform(occupancy[0], occupancy[1], n) if occupancy[0] != occupancy[1] else np.full(n, occupancy[0])
    mult = np.full(n, sg.n_total, dtype=np.int32)
    lcs = np.stack([random_rotation(rng, improper_lcs) for _ in range(n)])
    if hkl is None:
        hkl = unique_hkl(cell, sg, d_min=d_min, stol_max=stol_max)
    dtdf = rng.normal(size=len(hkl)) + 1j * rng.normal(size=len(hkl))
    anomalous = None
    if anomalous_per_atom:
        anomalous = rng.uniform(0, 0.2, n) + 1j * rng.uniform(0, 0.2, n)
    return Structure(cell=tuple(float(v) for v in cell), sg=sg, xyz=xyz, adp=adp, occupancy=occ,
                     multiplicity=mult, atom_wfn=atom_wfn, atom_type=atom_type, lcs=lcs,
                     wfns=wfns, types=types, hkl=np.asarray(hkl, dtype=np.int32), dtdf=dtdf,
                     anomalous=anomalous, name=name)


def protein_elements(n, rng):
    # C:N:O:S:H roughly as in proteins (with riding H)
    p = np.array([0.32, 0.085, 0.10, 0.005, 0.49])
    sym = np.array(["C", "N", "O", "S", "H"])
    e = rng.choice(sym, size=n, p=p / p.sum())
    e[:4] = ["C", "N", "O", "S"]
    return [str(v) for v in e]


def config0(seed=0):
    rng = np.random.default_rng(seed)
    cell = random_cell(rng, "monoclinic")
    elements = ["C"] * 12 + ["H"] * 12 + ["N"] * 4 + ["O"] * 4
    return build_structure(cell=cell, sg_symbol="P21/c", elements=elements, rng=rng,
                           stol_max=0.8, aniso=True, name="config0")


def config1(seed=1, n_atoms=5000, d_min=1.5, hkl=None):
    rng = np.random.default_rng(seed)
    cell = (60.0, 70.0, 80.0, 90.0, 90.0, 90.0)
    return build_structure(cell=cell, sg_symbol="P212121", elements=protein_elements(n_atoms, rng),
                           rng=rng, n_types=150, d_min=d_min, iso_b=(10.0, 40.0), hkl=hkl,
                           name="config1")


def config2(seed=2, n_atoms=50000, d_min=1.2, hkl=None):
    rng = np.random.default_rng(seed)
    cell = (120.0, 120.0, 140.0, 90.0, 90.0, 90.0)
    return build_structure(cell=cell, sg_symbol="P43212", elements=protein_elements(n_atoms, rng),
                           rng=rng, n_types=300, d_min=d_min, aniso=True, hkl=hkl, name="config2")


def small_case(sg_symbol="P21/c", n_atoms=6, stol_max=0.5, seed=7, cell_kind=None, **kw):
    rng = np.random.default_rng(seed)
    if cell_kind is None:
        cell_kind = {"P1": "triclinic", "P-1": "triclinic", "P-1(shift)": "triclinic",
                     "P21": "monoclinic", "P21/c": "monoclinic", "C2/c": "monoclinic",
                     "I2/m-like": "monoclinic", "R-3": "hexagonal", "P3": "hexagonal",
                     "R3(reverse)": "hexagonal"}.get(sg_symbol, "orthorhombic")
    cell = random_cell(rng, cell_kind)
    if sg_symbol in ("P43212", "P41"):
        a = cell[0]
        cell = (a, a, cell[2], 90.0, 90.0, 90.0)
    base = ["C", "H", "N", "O", "S"]
    elements = [base[i % len(base)] for i in range(n_atoms)]
    return build_structure(cell=cell, sg_symbol=sg_symbol, elements=elements, rng=rng,
                           stol_max=stol_max, name=f"small-{sg_symbol}", **kw)


# ---------------------------------------------------------------------------
# config 4: a batch of crystals with tabulated form factors
# ---------------------------------------------------------------------------
def config4_specs(n_crystals=256, seed=4):
    """(n_atoms, n_hkl) per crystal: atoms log-uniform in [10, 2000], reflections
    log-uniform in [2000, 100000]."""
    rng = np.random.default_rng(seed)
    atoms = np.exp(rng.uniform(math.log(10), math.log(2000), n_crystals)).astype(int)
    hkl = np.exp(rng.uniform(math.log(2000), math.log(100000), n_crystals)).astype(int)
    return [(int(a), int(h)) for a, h in zip(atoms, hkl)]


def config4_crystal(n_atoms, n_hkl, seed):
    """One crystal of the batch: P2_1/c, anisotropic ADPs (hydrogen isotropic),
    a cell of about 18 A^3 per atom, and the n_hkl unique reflections of lowest
    resolution (a complete sphere in sin(theta)/lambda, trimmed to n_hkl)."""
    rng = np.random.default_rng(seed)
    sg = space_group("P21/c")
    vol = 18.0 * n_atoms * sg.n_total
    beta = rng.uniform(95, 110)
    ratios = rng.uniform(0.8, 1.25, 3)
    edge = (vol / (np.prod(ratios) * math.sin(math.radians(beta)))) ** (1 / 3)
    cell = (edge * ratios[0], edge * ratios[1], edge * ratios[2], 90.0, beta, 90.0)
    # unique reflections ~ (4 pi / 3) V / d^3 / 4 for Laue class 2/m; ask for 30% more, keep the n_hkl lowest
    d = (4.0 * math.pi / 3.0 * vol / (4.0 * n_hkl * 1.3)) ** (1 / 3)
    while True:
        hkl = unique_hkl(cell, sg, d_min=d)
        if len(hkl) >= n_hkl:
            break
        d *= 0.9
    b = frac_to_cart_matrix(cell)
    binv = np.linalg.inv(b).T  # reciprocal basis
    s2 = np.sum((np.asarray(hkl, dtype=np.float64) @ binv.T) ** 2, axis=1)
    hkl = np.asarray(hkl)[np.argsort(s2, kind="stable")[:n_hkl]]
    elements = [("C", "N", "O", "H")[i] for i in rng.choice(4, n_atoms, p=[0.35, 0.1, 0.1, 0.45])]
    return build_structure(cell=cell, sg_symbol="P21/c", elements=elements, rng=rng, n_types=4, hkl=hkl,
                           aniso=True, l_max=0, name=f"config4-{seed}")


# per-element spherical f0(s) = Z sum_i w_i exp(-b_i s^2), s = sin(theta)/lambda, weights summing to one
# (Z electrons at s = 0, falling off like the core + valence densities above)
_F0 = {"H": (1, (0.5, 0.3, 0.2), (10.0, 25.0, 3.0)),
       "C": (6, (0.4, 0.3, 0.3), (20.0, 8.0, 0.5)),
       "N": (7, (0.4, 0.3, 0.3), (16.0, 6.5, 0.4)),
       "O": (8, (0.4, 0.3, 0.3), (13.0, 5.0, 0.3))}


def config4_f0_elements(st, s):
    """f0 per (reflection, element) at sin(theta)/lambda s [n_hkl], and the
    element index of every atom."""
    labels = sorted({st.wfns[w].label for w in st.atom_wfn})
    s2 = np.asarray(s, dtype=np.float64) ** 2
    f0 = np.zeros((len(s2), len(labels)))
    for j, e in enumerate(labels):
        z, ww, bb = _F0.get(e, _F0["C"])
        f0[:, j] = z * sum(wi * np.exp(-bi * s2) for wi, bi in zip(ww, bb))
    idx = {e: j for j, e in enumerate(labels)}
    return f0, np.array([idx[st.wfns[w].label] for w in st.atom_wfn], dtype=np.int64)


def config4_stol(st):
    """sin(theta)/lambda of every reflection of a crystal."""
    b = frac_to_cart_matrix(st.cell)
    binv = np.linalg.inv(b).T
    return 0.5 * np.linalg.norm(np.asarray(st.hkl, dtype=np.float64) @ binv.T, axis=1)


def config4_table(st, rng, n_ops=4):
    """A host table [n_hkl][n_ops][n_atoms] (complex128): f0 (1 + 0.05 CN(0, 1))
    (the tests' small crystals; the benchmark draws the same on the device)."""
    f0e, el = config4_f0_elements(st, config4_stol(st))
    f0 = f0e[:, el][:, None, :]
    shape = (st.n_hkl, n_ops, st.n_atoms)
    noise = (rng.normal(size=shape) + 1j * rng.normal(size=shape)) * (0.05 / math.sqrt(2.0))
    return f0 * (1.0 + noise)


# ---------------------------------------------------------------------------
# config 3: a served stream of refinement requests
# ---------------------------------------------------------------------------
CONFIG3_GROUPS = ("P1", "P-1", "P21", "P21/c", "P212121", "C2/c")


def config3_specs(n_structures=400, seed=3):
    """(n_atoms, n_hkl, space group) per structure: atoms log-uniform in
    [20, 20000], reflections log-uniform in [1000, 300000], the space group
    uniform over P1, P-1, P2_1, P2_1/c, P2_1 2_1 2_1, C2/c."""
    rng = np.random.default_rng(seed)
    atoms = np.exp(rng.uniform(math.log(20), math.log(20000), n_structures)).astype(int)
    hkl = np.exp(rng.uniform(math.log(1000), math.log(300000), n_structures)).astype(int)
    groups = rng.integers(len(CONFIG3_GROUPS), size=n_structures)
    return [(int(a), int(h), CONFIG3_GROUPS[g]) for a, h, g in zip(atoms, hkl, groups)]


def config3_structure(n_atoms, n_hkl, sg_symbol, seed):
    """One served structure, parameters as config0 (Hansen-Coppens multipoles
    to l = 4, anisotropic non-H atoms) with min(n_atoms, 64) shared types; a
    cell of about 18 A^3 per atom and the n_hkl lowest-resolution unique
    reflections."""
    rng = np.random.default_rng(seed)
    sg = space_group(sg_symbol)
    vol = 18.0 * n_atoms * sg.n_total
    kind = {"P1": "triclinic", "P-1": "triclinic"}.get(sg_symbol,
                                                       "orthorhombic" if sg_symbol == "P212121" else "monoclinic")
    angles = {"triclinic": (rng.uniform(80, 100), rng.uniform(95, 110), rng.uniform(80, 100)),
              "monoclinic": (90.0, rng.uniform(95, 110), 90.0), "orthorhombic": (90.0, 90.0, 90.0)}[kind]
    ratios = rng.uniform(0.8, 1.25, 3)
    unit = random_cell(rng, kind)  # consume the same draws as the small cases
    del unit
    cell0 = (1.0, 1.0, 1.0) + tuple(angles)
    v1 = abs(np.linalg.det(frac_to_cart_matrix(cell0)))
    edge = (vol / (np.prod(ratios) * v1)) ** (1 / 3)
    cell = tuple(edge * ratios) + tuple(angles)
    d = (4.0 * math.pi / 3.0 * vol / (max(2, sg.n_total) * n_hkl * 1.3)) ** (1 / 3)
    while True:
        hkl = unique_hkl(cell, sg, d_min=d)
        if len(hkl) >= n_hkl:
            break
        d *= 0.9
    b = frac_to_cart_matrix(cell)
    binv = np.linalg.inv(b).T
    s2 = np.sum((np.asarray(hkl, dtype=np.float64) @ binv.T) ** 2, axis=1)
    hkl = np.asarray(hkl)[np.argsort(s2, kind="stable")[:n_hkl]]
    elements = [("C", "N", "O", "H")[i] for i in rng.choice(4, n_atoms, p=[0.35, 0.1, 0.1, 0.45])]
    elements[:3] = ["C", "N", "O"][:min(3, n_atoms)]
    return build_structure(cell=cell, sg_symbol=sg_symbol, elements=elements, rng=rng,
                           n_types=min(n_atoms, 64), hkl=hkl, aniso=True, name=f"config3-{seed}")
