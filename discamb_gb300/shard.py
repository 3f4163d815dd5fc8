"""One structure's reflections sharded over several GPUs, one process per GPU.

F(h) is independent per reflection, so the reflection set splits across
ranks with no exchange during the sum.  Every rank holds the whole structure
(atoms, model, tables for its own reflections) and a contiguous share of the
reflections in line order: shares are cut only where a lattice line (h, k
fixed, l consecutive) ends, so each rank's engine keeps its line recurrences
whole.  Each rank computes F of its share and its partial sums of the
per-atom derivatives; one all-reduce (sum) of the derivative vector (n_atoms
x up to 38 channels, 15 MB for 50,000 atoms) gives every rank the gradient
of the whole set.  F stays with the rank that computed it, or is gathered
into the caller's order on request.

The reference computes one structure on one machine with OpenMP threads over
contiguous shares of its line-ordered reflections
(scattering_utilities::splitHklLines, src/Scattering/scattering_utilities.cpp:
463-517, merged by merge_dTarget_dParameterSets, :236-267); the ranks here
take the place of its threads, the all-reduce that of its merge.
"""
from __future__ import annotations

import numpy as np

# derivative outputs of one call, in the order of the reduced vector
_CHANNELS = (("d_xyz", 3), ("d_adp", 6), ("d_occ", 1), ("d_pval", 1), ("d_plm", 25), ("d_kappa", 1),
             ("d_kappa_p", 1))


def line_order(hkl):
    """Indices of hkl sorted in line order (h, then k, then l)."""
    hkl = np.asarray(hkl, dtype=np.int64).reshape(-1, 3)
    return np.lexsort((hkl[:, 2], hkl[:, 1], hkl[:, 0]))


def shard_indices(hkl, world):
    """Per rank, the caller-order indices of its reflections: contiguous
    shares of the line-ordered set of about n / world reflections each,
    every cut moved forward to the next line start (a line is a run of
    reflections with the same h, k and consecutive l).  Every reflection is
    in exactly one share; a share may be empty when lines are long and the
    set is small."""
    hkl = np.asarray(hkl, dtype=np.int64).reshape(-1, 3)
    n = len(hkl)
    order = line_order(hkl)
    s = hkl[order]
    starts = np.ones(n, dtype=bool)
    if n > 1:
        cont = (s[1:, 0] == s[:-1, 0]) & (s[1:, 1] == s[:-1, 1]) & (s[1:, 2] == s[:-1, 2] + 1)
        starts[1:] = ~cont
    line_start = np.flatnonzero(starts)
    cuts = [0]
    for r in range(1, world):
        target = (n * r) // world
        j = np.searchsorted(line_start, max(target, cuts[-1]))
        cuts.append(int(line_start[j]) if j < len(line_start) else n)
    cuts.append(n)
    return [order[cuts[r]:cuts[r + 1]] for r in range(world)]


def derivative_vector(result, n_atoms):
    """The derivative outputs of one call as one float64 vector (the order
    of _CHANNELS; channels the result lacks are left out) and the layout."""
    parts, layout = [], []
    for key, width in _CHANNELS:
        if key not in result:
            continue
        v = result[key]
        if isinstance(v, list):  # per-atom ADP lists: padded to six
            pad = np.zeros((n_atoms, width))
            for i, a in enumerate(v):
                pad[i, :len(a)] = a
            v = pad
        v = np.asarray(v, dtype=np.float64).reshape(n_atoms, -1)
        parts.append(v.reshape(-1))
        layout.append((key, v.shape[1]))
    return np.concatenate(parts) if parts else np.zeros(0), layout


def split_vector(vec, layout, n_atoms, n_adp=None):
    """The inverse of derivative_vector; d_adp back to per-atom lists when
    n_adp (component counts) is given."""
    out, o = {}, 0
    for key, width in layout:
        block = vec[o:o + n_atoms * width].reshape(n_atoms, width)
        o += n_atoms * width
        if key == "d_adp" and n_adp is not None:
            out[key] = [block[i, :n_adp[i]].copy() for i in range(n_atoms)]
        elif width == 1:
            out[key] = block[:, 0].copy()
        else:
            out[key] = block.copy()
    return out


class ShardedCalculator:
    """A structure's calculation with its reflections sharded over the ranks
    of a torch.distributed process group (NCCL on GPUs, gloo on CPU).

    make(hkl_share) -> a calculator of this rank's reflections whose
    calculate(dtdf_share, **kw) returns F and the per-atom derivative sums of
    those reflections (an engine calculator of this package).  calculate()
    returns the whole set's derivatives on every rank and, with gather_f,
    F of every reflection in the caller's order (else this rank's share and
    its caller-order indices)."""

    def __init__(self, make, hkl, n_atoms, n_adp=None, group=None, device=None):
        import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.world = dist.get_world_size(group)
        self.rank = dist.get_rank(group)
        self.n_hkl = len(hkl)
        self.n_atoms = n_atoms
        self.n_adp = n_adp
        self.device = device
        self.shares = shard_indices(hkl, self.world)
        self.idx = self.shares[self.rank]
        self.calc = make(np.asarray(hkl)[self.idx]) if len(self.idx) else None

    def calculate(self, dtdf, gather_f=True, **kw):
        import torch
        dist = self.dist
        dtdf = np.asarray(dtdf)
        r = self.calc.calculate(dtdf[self.idx], **kw) if self.calc is not None else None
        if r is None:  # an empty share still takes part in the collectives
            r = {"f": np.zeros(0, dtype=np.complex128)}
            for key, width in _CHANNELS[:3]:
                r[key] = np.zeros((self.n_atoms, width)) if width > 1 else np.zeros(self.n_atoms)
        vec, layout = derivative_vector(r, self.n_atoms)
        t = torch.from_numpy(vec.copy())
        if self.device is not None:
            t = t.to(self.device)
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=self.group)  # the one exchange of the path
        out = split_vector(t.cpu().numpy(), layout, self.n_atoms, self.n_adp)
        f = np.asarray(r["f"], dtype=np.complex128)
        if not gather_f:
            out["f"], out["f_indices"] = f, self.idx
            return out
        # F of every share, padded to the longest, gathered and put back in the caller's order
        m = max(len(s) for s in self.shares)
        buf = np.zeros((m, 2))
        buf[:len(f), 0], buf[:len(f), 1] = f.real, f.imag
        mine = torch.from_numpy(buf)
        if self.device is not None:
            mine = mine.to(self.device)
        parts = [torch.zeros_like(mine) for _ in range(self.world)]
        dist.all_gather(parts, mine, group=self.group)
        full = np.zeros(self.n_hkl, dtype=np.complex128)
        for s, p in zip(self.shares, parts):
            p = p.cpu().numpy()
            full[s] = p[:len(s), 0] + 1j * p[:len(s), 1]
        out["f"] = full
        return out
