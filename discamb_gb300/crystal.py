"""Host-side crystallography for the structure-factor path.

Cell matrices, space-group decomposition into the engine's symmetry subset,
centering multipliers, unique-reflection generation and ADP / coordinate
convention conversions.  All of it is O(n_atoms + n_hkl) host work that the
reference also keeps on the host:

* cell matrices follow ``UnitCell::calculateTransformationMatrices``
  (src/CrystalStructure/UnitCell.cpp:183-212): a along x, b in the xy plane;
* the reciprocal basis follows ``ReciprocalLatticeUnitCell::set``
  (src/CrystalStructure/ReciprocalLatticeUnitCell.cpp:27-51);
* the symmetry subset (operations modulo inversion and lattice centering) is
  what ``HansenCoppensStructureFactorCalculator::setEngineSpecificSpaceGroup
  Representation`` feeds the CPU engine
  (src/Scattering/HansenCoppensStructureFactorCalculator.cpp:107-155);
* centering multipliers follow ``scattering_utilities::centeringSfMultipliers``
  (src/Scattering/scattering_utilities.cpp:103-170);
* ADP conventions follow ``StructuralParametersConverter``
  (src/CrystalStructure/StructuralParametersConverter.cpp:28-95).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from fractions import Fraction
import itertools
import math

import numpy as np

# ---------------------------------------------------------------------------
# cell
# ---------------------------------------------------------------------------


def frac_to_cart_matrix(cell):
    """M with r_cart = M r_frac (a along x, b in the xy plane)."""
    a, b, c, al, be, ga = [float(v) for v in cell]
    f = math.pi / 180.0
    ca, cb, cg, sg = math.cos(al * f), math.cos(be * f), math.cos(ga * f), math.sin(ga * f)
    phi = math.sqrt(1 - ca * ca - cb * cb - cg * cg + 2 * ca * cb * cg)
    m = np.zeros((3, 3))
    m[0, 0] = a
    m[0, 1] = b * cg
    m[0, 2] = c * cb
    m[1, 1] = b * sg
    m[1, 2] = (c / sg) * (ca - cb * cg)
    m[2, 2] = c * phi / sg
    return m


def reciprocal_matrix(cell):
    """B with h_cart = B h_frac; columns are a*, b*, c* in the Cartesian frame."""
    m = frac_to_cart_matrix(cell)
    a, b, c = m[:, 0], m[:, 1], m[:, 2]
    v = np.dot(np.cross(a, b), c)
    bm = np.zeros((3, 3))
    bm[:, 0] = np.cross(b, c) / v
    bm[:, 1] = np.cross(c, a) / v
    bm[:, 2] = np.cross(a, b) / v
    return bm


# ---------------------------------------------------------------------------
# symmetry operations
# ---------------------------------------------------------------------------

_AXES = {"x": 0, "y": 1, "z": 2}


def parse_symop(text):
    """'-x+1/2,y,-z+3/4' -> (R int 3x3, t as 3 Fractions); x' = R x + t."""
    rows = text.replace(" ", "").lower().split(",")
    if len(rows) != 3:
        raise ValueError(f"bad symmetry operation '{text}'")
    rot = np.zeros((3, 3), dtype=np.int64)
    trans = []
    for i, row in enumerate(rows):
        t = Fraction(0)
        tok = ""
        sign = 1
        j = 0
        row = row + "+"
        while j < len(row):
            ch = row[j]
            if ch in "+-":
                if tok:
                    if tok in _AXES:
                        rot[i, _AXES[tok]] += sign
                    else:
                        t += sign * Fraction(tok)
                tok = ""
                sign = 1 if ch == "+" else -1
            else:
                tok += ch
            j += 1
        trans.append(t % 1)
    return rot, tuple(trans)


def _t12(t):
    """translation as integers in units of 1/12 (mod 12)."""
    out = []
    for v in t:
        q = Fraction(v) * 12
        if q.denominator != 1:
            raise ValueError("translation not a multiple of 1/12")
        out.append(int(q) % 12)
    return tuple(out)


def _compose(op1, op2):
    """op1 o op2 (apply op2 first)."""
    r1, t1 = op1
    r2, t2 = op2
    r = r1 @ r2
    t = tuple(int((np.dot(r1[i], t2) + t1[i])) % 12 for i in range(3))
    return r, t


@dataclass
class SpaceGroup:
    """A space group given by its full list of operations, decomposed the way
    the reference engine consumes it."""

    symbol: str
    ops_text: list
    rot: np.ndarray = field(init=False)          # (n_total,3,3) int, all ops
    trans12: np.ndarray = field(init=False)      # (n_total,3) int, units 1/12
    subset_rot: np.ndarray = field(init=False)   # (n_sub,3,3) engine subset
    subset_trans: np.ndarray = field(init=False)  # (n_sub,3) float fractional
    centrosymmetric: bool = field(init=False)
    inversion_translation: np.ndarray = field(init=False)  # fractional t of -x+t
    centering: str = field(init=False)
    obverse: bool = field(init=False)

    def __post_init__(self):
        parsed = [parse_symop(s) for s in self.ops_text]
        ops = [(r, _t12(t)) for r, t in parsed]
        # closure check: the list must be a group modulo lattice translations
        keys = {(r.tobytes(), t) for r, t in ops}
        for a, b in itertools.product(ops, ops):
            r, t = _compose(a, b)
            if (r.tobytes(), t) not in keys:
                raise ValueError(f"operations of {self.symbol} are not closed")
        self.rot = np.array([r for r, _ in ops], dtype=np.int64)
        self.trans12 = np.array([t for _, t in ops], dtype=np.int64)
        ident = np.eye(3, dtype=np.int64)
        cvecs = [t for r, t in ops if np.array_equal(r, ident)]
        self._cvecs = cvecs
        self.centering, self.obverse = _centering_letter(cvecs)
        inv = [t for r, t in ops if np.array_equal(r, -ident)]
        self.centrosymmetric = bool(inv)
        t_inv = min(inv) if inv else (0, 0, 0)
        self.inversion_translation = np.array(t_inv, dtype=np.float64) / 12.0
        # subset: one representative per coset of {centering} x {1, inversion}
        chosen = []
        seen = set()
        for r, t in ops:
            key = (r.tobytes(), t)
            if key in seen:
                continue
            chosen.append((r, t))
            for c in cvecs:
                tc = tuple((t[i] + c[i]) % 12 for i in range(3))
                seen.add((r.tobytes(), tc))
                if self.centrosymmetric:
                    ti = tuple((t_inv[i] - tc[i]) % 12 for i in range(3))
                    seen.add(((-r).tobytes(), ti))
        self.subset_rot = np.array([r for r, _ in chosen], dtype=np.int64)
        self.subset_trans = np.array([t for _, t in chosen], dtype=np.float64) / 12.0

    @property
    def n_total(self):
        return len(self.rot)

    @property
    def n_subset(self):
        return len(self.subset_rot)

    @property
    def point_group_order(self):
        """Operations counted by the throughput metric: point-group order
        without lattice centering (subset x 2 for centrosymmetric groups)."""
        return self.n_subset * (2 if self.centrosymmetric else 1)

    def all_trans(self):
        return self.trans12.astype(np.float64) / 12.0


def _centering_letter(cvecs):
    s = {tuple(v) for v in cvecs}
    s.discard((0, 0, 0))
    if not s:
        return "P", True
    if s == {(6, 6, 0)}:
        return "C", True
    if s == {(0, 6, 6)}:
        return "A", True
    if s == {(6, 0, 6)}:
        return "B", True
    if s == {(6, 6, 6)}:
        return "I", True
    if s == {(6, 6, 0), (0, 6, 6), (6, 0, 6)}:
        return "F", True
    if s == {(8, 4, 4), (4, 8, 8)}:
        return "R", True
    if s == {(4, 8, 4), (8, 4, 8)}:
        return "R", False
    raise ValueError(f"unsupported centering translations {s}")


SPACE_GROUPS = {
    "P1": ["x,y,z"],
    "P-1": ["x,y,z", "-x,-y,-z"],
    "P21": ["x,y,z", "-x,y+1/2,-z"],
    "P21/c": ["x,y,z", "-x,y+1/2,-z+1/2", "-x,-y,-z", "x,-y+1/2,z+1/2"],
    "P212121": ["x,y,z", "-x+1/2,-y,z+1/2", "-x,y+1/2,-z+1/2", "x+1/2,-y+1/2,-z"],
    "C2/c": ["x,y,z", "-x,y,-z+1/2", "-x,-y,-z", "x,-y,z+1/2",
             "x+1/2,y+1/2,z", "-x+1/2,y+1/2,-z+1/2", "-x+1/2,-y+1/2,-z", "x+1/2,-y+1/2,z+1/2"],
    "P43212": ["x,y,z", "-x,-y,z+1/2", "-y+1/2,x+1/2,z+3/4", "y+1/2,-x+1/2,z+1/4",
               "-x+1/2,y+1/2,-z+3/4", "x+1/2,-y+1/2,-z+1/4", "y,x,-z", "-y,-x,-z+1/2"],
    "P41": ["x,y,z", "-x,-y,z+1/2", "-y,x,z+1/4", "y,-x,z+3/4"],
    "Pbca": ["x,y,z", "-x+1/2,-y,z+1/2", "-x,y+1/2,-z+1/2", "x+1/2,-y+1/2,-z",
             "-x,-y,-z", "x+1/2,y,-z+1/2", "x,-y+1/2,z+1/2", "-x+1/2,y+1/2,z"],
    # inversion centre away from the origin (exercises the shifted-centre branch)
    "P-1(shift)": ["x,y,z", "-x+1/2,-y,-z+1/2"],
    "I2/m-like": ["x,y,z", "-x,y,-z", "-x,-y,-z", "x,-y,z",
                  "x+1/2,y+1/2,z+1/2", "-x+1/2,y+1/2,-z+1/2", "-x+1/2,-y+1/2,-z+1/2",
                  "x+1/2,-y+1/2,z+1/2"],
}


def _with_centering(ops, vectors):
    """Every operation of ``ops`` combined with every centering translation
    (fractions as text, e.g. ("2/3", "1/3", "1/3"))."""
    out = []
    for v in [("0", "0", "0")] + list(vectors):
        for op in ops:
            rows = op.split(",")
            out.append(",".join(r if t == "0" else f"{r}+{t}" for r, t in zip(rows, v)))
    return out


_R_OBVERSE = [("2/3", "1/3", "1/3"), ("1/3", "2/3", "2/3")]
_R_REVERSE = [("1/3", "2/3", "1/3"), ("2/3", "1/3", "2/3")]
_F_VECTORS = [("0", "1/2", "1/2"), ("1/2", "0", "1/2"), ("1/2", "1/2", "0")]
_P3 = ["x,y,z", "-y,x-y,z", "-x+y,-x,z"]
_P3_INV = ["-x,-y,-z", "y,-x+y,-z", "x-y,x,-z"]
SPACE_GROUPS.update({
    "P3": list(_P3),
    # rhombohedral centering on hexagonal axes, obverse and reverse settings
    "R-3": _with_centering(_P3 + _P3_INV, _R_OBVERSE),
    "R3(reverse)": _with_centering(_P3, _R_REVERSE),
    # face centering with quarter-cell glide translations
    "Fdd2": _with_centering(["x,y,z", "-x,-y,z", "x+1/4,-y+1/4,z+1/4", "-x+1/4,y+1/4,z+1/4"], _F_VECTORS),
})


def space_group(symbol):
    return SpaceGroup(symbol, SPACE_GROUPS[symbol])


def centering_multipliers(centering, obverse, hkl):
    """Per-reflection lattice-centering multiplier (0 for absences)."""
    hkl = np.asarray(hkl, dtype=np.int64)
    h, k, l = hkl[:, 0], hkl[:, 1], hkl[:, 2]
    c = centering.upper()
    if c == "P":
        return np.ones(len(hkl))
    if c == "R":
        # obverse: -h + k + l = 3n.  Reverse: the reference tests (h - k + l) mod 2
        # (scattering_utilities.cpp:130), and so does this restatement
        if obverse:
            return np.where(np.abs(-h + k + l) % 3 == 0, 3.0, 0.0)
        return np.where(np.abs(h - k + l) % 2 == 0, 3.0, 0.0)
    if c == "F":
        hm, km, lm = np.abs(h % 2), np.abs(k % 2), np.abs(l % 2)
        return np.where((hm == km) & (hm == lm), 4.0, 0.0)
    if c == "I":
        s = h + k + l
    elif c == "A":
        s = k + l
    elif c == "B":
        s = h + l
    elif c == "C":
        s = h + k
    else:
        raise ValueError(f"centering '{centering}' not supported")
    return np.where(s % 2 == 0, 2.0, 0.0)


def unique_hkl(cell, sg: SpaceGroup, d_min=None, stol_max=None, drop_absent=True):
    """All reflections with d >= d_min (or sin(theta)/lambda <= stol_max), one
    per Laue-equivalent set (the lexicographically largest representative),
    without 000 and, optionally, without lattice-centering absences."""
    if stol_max is not None:
        d_min = 1.0 / (2.0 * stol_max)
    hmax_len = 1.0 / d_min
    bm = reciprocal_matrix(cell)
    g = bm.T @ bm
    # bounds: |h_i| <= hmax_len * |a_i|
    m = frac_to_cart_matrix(cell)
    lim = [int(math.floor(hmax_len * np.linalg.norm(m[:, i]))) + 1 for i in range(3)]
    rng = [np.arange(-L, L + 1) for L in lim]
    H, K, Lg = np.meshgrid(*rng, indexing="ij")
    hkl = np.stack([H.ravel(), K.ravel(), Lg.ravel()], axis=1)
    q = np.einsum("ni,ij,nj->n", hkl.astype(np.float64), g, hkl.astype(np.float64))
    keep = (q <= hmax_len * hmax_len * (1 + 1e-12)) & (np.abs(hkl).sum(axis=1) > 0)
    hkl = hkl[keep]
    # Laue group: rotation parts and their negatives acting as h -> R^T h
    rots = np.unique(sg.rot.reshape(-1, 9), axis=0).reshape(-1, 3, 3)
    laue = np.concatenate([rots, -rots])
    best = hkl.copy()
    for r in laue:
        cand = hkl @ r  # row vector h times R == (R^T h)^T
        # lexicographic max
        gt = (cand[:, 0] > best[:, 0]) | ((cand[:, 0] == best[:, 0]) & (
            (cand[:, 1] > best[:, 1]) | ((cand[:, 1] == best[:, 1]) & (cand[:, 2] > best[:, 2]))))
        best[gt] = cand[gt]
    is_rep = np.all(best == hkl, axis=1)
    hkl = hkl[is_rep]
    if drop_absent:
        mult = centering_multipliers(sg.centering, sg.obverse, hkl)
        hkl = hkl[mult != 0]
    order = np.lexsort((hkl[:, 2], hkl[:, 1], hkl[:, 0]))
    return np.ascontiguousarray(hkl[order].astype(np.int32))


# ---------------------------------------------------------------------------
# ADP and coordinate conventions
# ---------------------------------------------------------------------------

def _voigt_to_mat(u):
    u = np.asarray(u)
    m = np.empty(u.shape[:-1] + (3, 3))
    m[..., 0, 0], m[..., 1, 1], m[..., 2, 2] = u[..., 0], u[..., 1], u[..., 2]
    m[..., 0, 1] = m[..., 1, 0] = u[..., 3]
    m[..., 0, 2] = m[..., 2, 0] = u[..., 4]
    m[..., 1, 2] = m[..., 2, 1] = u[..., 5]
    return m


def _mat_to_voigt(m):
    return np.stack([m[..., 0, 0], m[..., 1, 1], m[..., 2, 2],
                     m[..., 0, 1], m[..., 0, 2], m[..., 1, 2]], axis=-1)


def adp_transform_matrix(cell, src, dst):
    """A with U_dst = A U_src A^T (U as symmetric 3x3), conventions
    'U_cif', 'U_cart', 'U_star'."""
    m = frac_to_cart_matrix(cell)
    bm = reciprocal_matrix(cell)
    lam = np.diag(np.linalg.norm(bm, axis=0))
    minv = np.linalg.inv(m)
    to_cart = {"U_cif": m @ lam, "U_cart": np.eye(3), "U_star": m}
    a_src = to_cart[src]
    a_dst_inv = np.linalg.inv(to_cart[dst])
    return a_dst_inv @ a_src


def convert_adp(cell, u, src, dst):
    if src == dst:
        return np.array(u, dtype=np.float64)
    a = adp_transform_matrix(cell, src, dst)
    return _mat_to_voigt(a @ _voigt_to_mat(u) @ a.T)


def convert_adp_gradient(cell, g, src, dst):
    """Gradient with respect to the six independent parameters
    (U11,U22,U33,U12,U13,U23) in convention ``src`` -> same in ``dst``."""
    if src == dst:
        return np.array(g, dtype=np.float64)
    g = np.array(g, dtype=np.float64)
    gm = _voigt_to_mat(g)
    gm[..., 0, 1] *= 0.5
    gm[..., 1, 0] *= 0.5
    gm[..., 0, 2] *= 0.5
    gm[..., 2, 0] *= 0.5
    gm[..., 1, 2] *= 0.5
    gm[..., 2, 1] *= 0.5
    # U_src = A_ds U_dst A_ds^T with A_ds mapping dst -> src
    a = adp_transform_matrix(cell, dst, src)
    out = a.T @ gm @ a
    out = _mat_to_voigt(out)
    out[..., 3:] *= 2.0
    return out


def convert_xyz_gradient(cell, g, src, dst):
    """d/d(frac) <-> d/d(cart): r_cart = M r_frac so d/dfrac = M^T d/dcart."""
    if src == dst:
        return np.array(g, dtype=np.float64)
    m = frac_to_cart_matrix(cell)
    g = np.asarray(g, dtype=np.float64)
    if src == "cartesian" and dst == "fractional":
        return g @ m
    if src == "fractional" and dst == "cartesian":
        return g @ np.linalg.inv(m)
    raise ValueError("unknown xyz convention")
