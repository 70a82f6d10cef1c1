"""Periodic Bravais lattices with a basis, and their directed bond lists.

Mirrors the lattice types the reference's HubbardModel is built on
(src/lattices/constructors.jl:1-72, src/lattices/lattice.jl:231-374).
Site numbering follows the reference's ``_sub2ind`` (lattice.jl:240-254):
for Bravais coordinates (x1, x2, ...) and basis index b, all 1-based,
``flat = x1 + L1*(x2-1) + L1*L2*(b-1)``.  Python indices here are 0-based,
so site ``flat - 1`` of the reference is index ``flat - 1`` here.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Sequence, Tuple


@dataclass(frozen=True)
class Bond:
    """Bond from basis site ``frm`` to basis site ``to`` (1-based), crossing
    ``uc_shift`` unit cells (reference ``Bond``, lattice.jl:38-45)."""

    frm: int
    to: int
    uc_shift: Tuple[int, ...]
    label: int = 1


@dataclass
class UnitCell:
    name: str
    lattice_vectors: Tuple[Tuple[float, ...], ...]
    sites: List[Tuple[float, ...]]
    bonds: List[Bond]


@dataclass
class Lattice:
    """A periodic lattice: unit cell repeated ``Ls`` times (reference ``Lattice``)."""

    unitcell: UnitCell
    Ls: Tuple[int, ...]
    _bonds: List[Tuple[int, int]] = field(default=None, repr=False)

    def __len__(self) -> int:
        return int(math.prod(self.Ls)) * len(self.unitcell.sites)

    @property
    def name(self) -> str:
        return self.unitcell.name

    def size(self) -> Tuple[int, ...]:
        return tuple(self.Ls)

    def _shift_bravais(self, idx: int, b: Bond) -> Tuple[int, int]:
        """Reference ``_shift_Bravais`` (lattice.jl:327-357); idx is 1-based
        Bravais index; returns 1-based (from, to) site indices."""
        flat_out = 1
        flat_fld = idx
        f = 1
        for d, L in enumerate(self.Ls):
            # fldmod1(flat_fld, L)
            q, r = divmod(flat_fld - 1, L)
            flat_fld, t = q + 1, r + 1
            t = (t - 1 + b.uc_shift[d]) % L + 1
            flat_out += f * (t - 1)
            f *= L
        return idx + (b.frm - 1) * f, flat_out + (b.to - 1) * f

    def bonds(self, directed: bool = True) -> List[Tuple[int, int]]:
        """All directed bonds as 0-based (from, to) pairs, in the reference's
        iteration order (``bonds(l, Val(true))``, lattice.jl:367-373)."""
        if not directed:
            raise NotImplementedError("only directed bond iteration is used by the DQMC path")
        if self._bonds is None:
            out = []
            for idx in range(1, int(math.prod(self.Ls)) + 1):
                for b in self.unitcell.bonds:
                    fr, to = self._shift_bravais(idx, b)
                    out.append((fr - 1, to - 1))
            self._bonds = out
        return self._bonds

    def n_bravais(self) -> int:
        return int(math.prod(self.Ls))

    def pair_distance_index(self):
        """Slot of every site pair (src, trg) in the by-distance arrays of the
        reference's EachSitePairByDistance (lattice_iterators.jl:160-168,
        generic.jl:434-461): output shape (Ndir, B, B) column-major with
        Ndir = Bravais sites, B = basis sites; the direction of a pair is the
        Bravais shift from src's cell to trg's, per dimension (trg - src) mod L
        flattened like _sub2ind (the Bravais dir2srctrg, lattice_cache.jl:
        226-242).  Returns an (n, n) int array, 0-based slots, [src, trg]."""
        import numpy as np

        nb, B = self.n_bravais(), len(self.unitcell.sites)
        n = nb * B
        coords = np.zeros((nb, len(self.Ls)), dtype=np.int64)
        for idx in range(nb):
            rem = idx
            for d, L in enumerate(self.Ls):
                coords[idx, d] = rem % L
                rem //= L
        shift = np.zeros((nb, nb), dtype=np.int64)
        stride = 1
        for d, L in enumerate(self.Ls):
            shift += ((coords[None, :, d] - coords[:, None, d]) % L) * stride
            stride *= L
        out = np.zeros((n, n), dtype=np.int32)
        for b1 in range(B):
            for b2 in range(B):
                out[b1 * nb:(b1 + 1) * nb, b2 * nb:(b2 + 1) * nb] = shift + nb * (b1 + B * b2)
        return out

    def positions(self):
        """Real-space site positions (n x dim), used for Fourier sums."""
        import numpy as np

        pos = []
        uc = self.unitcell
        nb = int(math.prod(self.Ls))
        for b, s in enumerate(uc.sites):
            for idx in range(nb):
                rem = idx
                r = list(s)
                for d, L in enumerate(self.Ls):
                    x = rem % L
                    rem //= L
                    r = [ri + x * vi for ri, vi in zip(r, uc.lattice_vectors[d])]
                pos.append(r)
        return np.asarray(pos, dtype=float)


def Chain(Lx: int) -> Lattice:
    uc = UnitCell("Chain", ((1.0,),), [(0.0,)], [Bond(1, 1, (1,)), Bond(1, 1, (-1,))])
    return Lattice(uc, (Lx,))


def SquareLattice(Lx: int, Ly: int = None) -> Lattice:
    Ly = Lx if Ly is None else Ly
    uc = UnitCell(
        "Square",
        ((1.0, 0.0), (0.0, 1.0)),
        [(0.0, 0.0)],
        [Bond(1, 1, (1, 0)), Bond(1, 1, (0, 1)), Bond(1, 1, (-1, 0)), Bond(1, 1, (0, -1))],
    )
    return Lattice(uc, (Lx, Ly))


def CubicLattice(Lx: int, Ly: int = None, Lz: int = None) -> Lattice:
    Ly = Lx if Ly is None else Ly
    Lz = Lx if Lz is None else Lz
    uc = UnitCell(
        "Cubic",
        ((1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0)),
        [(0.0, 0.0, 0.0)],
        [
            Bond(1, 1, (1, 0, 0)), Bond(1, 1, (0, 1, 0)), Bond(1, 1, (0, 0, 1)),
            Bond(1, 1, (-1, 0, 0)), Bond(1, 1, (0, -1, 0)), Bond(1, 1, (0, 0, -1)),
        ],
    )
    return Lattice(uc, (Lx, Ly, Lz))


def Honeycomb(Lx: int, Ly: int = None) -> Lattice:
    Ly = Lx if Ly is None else Ly
    s3 = math.sqrt(3.0)
    uc = UnitCell(
        "Honeycomb",
        ((s3 / 2, -0.5), (s3 / 2, 0.5)),
        [(0.0, 0.0), (1 / s3, 0.0)],
        [
            Bond(1, 2, (0, 0)), Bond(1, 2, (-1, 0)), Bond(1, 2, (0, -1)),
            Bond(2, 1, (0, 0)), Bond(2, 1, (1, 0)), Bond(2, 1, (0, 1)),
        ],
    )
    return Lattice(uc, (Lx, Ly))


def TriangularLattice(Lx: int, Ly: int = None) -> Lattice:
    Ly = Lx if Ly is None else Ly
    s3 = math.sqrt(3.0)
    uc = UnitCell(
        "Triangular",
        ((s3 / 2, -0.5), (s3 / 2, 0.5)),
        [(0.0, 0.0)],
        [
            Bond(1, 1, (1, 0)), Bond(1, 1, (0, 1)), Bond(1, 1, (-1, 1)),
            Bond(1, 1, (-1, 0)), Bond(1, 1, (0, -1)), Bond(1, 1, (1, -1)),
        ],
    )
    return Lattice(uc, (Lx, Ly))


def choose_lattice(dims: int, L: int) -> Lattice:
    """``choose_lattice`` of HubbardModel.jl:58-66."""
    if dims == 1:
        return Chain(L)
    if dims == 2:
        return SquareLattice(L)
    return CubicLattice(*([L] * dims))
