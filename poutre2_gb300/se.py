"""Structuring-element vocabulary, mirroring poutre2's ``structuring_element`` module.

* ``Common_NL_SE`` / ``Compound_NL_SE``: the predefined static SEs
  (include/poutre/structuring_element/se_types_and_tags.hpp:45-63).
* ``NeighborList``: an explicit offset list, the runtime ``neighbor_list_t<Rank>``
  (include/poutre/structuring_element/details/neighbor_list_se_t.hpp:36-228).
* ``predefined_offsets``: the predefined runtime neighbour lists
  (src/structuring_element/predefined_nl_se.cpp:19-92), centre first, same order.

Offsets are tuples in reference coordinate order (d0 slowest ... d_{rank-1} fastest),
i.e. (dy, dx) for images and (dz, dy, dx) for volumes.
"""
from __future__ import annotations

import enum
from typing import Iterable, List, Sequence, Tuple


class Common_NL_SE(enum.IntEnum):
    Undef = 0
    SESegmentX1D = 1
    SESquare2D = 2
    SECross2D = 3
    SESegmentX2D = 4
    SESegmentY2D = 5
    SESegmentX3D = 6
    SESegmentY3D = 7
    SESegmentZ3D = 8
    SECross3D = 9
    SESquare3D = 10


class Compound_NL_SE(enum.IntEnum):
    Undef = 0
    Octagon = 1
    Rhombicuboctahedron = 2


SE_RANK = {
    Common_NL_SE.SESegmentX1D: 1,
    Common_NL_SE.SESquare2D: 2, Common_NL_SE.SECross2D: 2,
    Common_NL_SE.SESegmentX2D: 2, Common_NL_SE.SESegmentY2D: 2,
    Common_NL_SE.SESegmentX3D: 3, Common_NL_SE.SESegmentY3D: 3, Common_NL_SE.SESegmentZ3D: 3,
    Common_NL_SE.SECross3D: 3, Common_NL_SE.SESquare3D: 3,
}

_PREDEFINED = {
    "SESegmentX1D": [(0,), (-1,), (1,)],
    "SESegmentX2D": [(0, 0), (0, -1), (0, 1)],
    "SESegmentY2D": [(0, 0), (-1, 0), (1, 0)],
    "SESquare2D": [(0, 0), (-1, -1), (0, -1), (1, -1), (-1, 0), (1, 0), (-1, 1), (0, 1), (1, 1)],
    "SECross2D": [(0, 0), (0, -1), (-1, 0), (1, 0), (0, 1)],
    "SECross3D": [(0, 0, 0), (0, 0, -1), (0, -1, 0), (-1, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)],
    "SESquare3D": [(0, 0, 0)] + [(a, b, c) for c in (-1, 0, 1) for b in (-1, 0, 1) for a in (-1, 0, 1)
                                 if (a, b, c) != (0, 0, 0)],
    "SESegmentX3D": [(0, 0, 0), (0, 0, -1), (0, 0, 1)],
    "SESegmentY3D": [(0, 0, 0), (0, -1, 0), (0, 1, 0)],
    "SESegmentZ3D": [(0, 0, 0), (-1, 0, 0), (1, 0, 0)],
}


def predefined_offsets(name) -> List[Tuple[int, ...]]:
    """Offsets of a predefined runtime SE (``poutre::se::SESquare2D`` ...)."""
    if isinstance(name, Common_NL_SE):
        name = name.name
    return list(_PREDEFINED[name])


class NeighborList:
    """Explicit offset-list SE (``neighbor_list_t<Rank>``)."""

    def __init__(self, offsets: Iterable[Sequence[int]]):
        offs = [tuple(int(v) for v in o) for o in offsets]
        if not offs:
            raise ValueError("empty neighbour list")
        rank = len(offs[0])
        if rank < 1 or rank > 3 or any(len(o) != rank for o in offs):
            raise ValueError("offsets must all have the same rank in [1,3]")
        self.offsets = offs
        self.rank = rank

    @classmethod
    def predefined(cls, name) -> "NeighborList":
        return cls(predefined_offsets(name))

    @classmethod
    def segment(cls, dy: int, dx: int, half: int) -> "NeighborList":
        """Line segment t*(dy,dx), t in [-half, half], centre first (e.g. the 45-degree
        segment is ``segment(-1, 1, 31)`` = offsets (-t, +t))."""
        return cls([(0, 0)] + [(t * dy, t * dx) for t in range(-half, half + 1) if t != 0])

    @classmethod
    def rectangle(cls, hy: int, hx: int) -> "NeighborList":
        return cls([(0, 0)] + [(y, x) for y in range(-hy, hy + 1) for x in range(-hx, hx + 1) if (y, x) != (0, 0)])

    # neighbor_list_t API (neighbor_list_se_t.hpp)
    def GetSize(self) -> int:
        return len(self.offsets)

    def Transpose(self) -> "NeighborList":
        return NeighborList([tuple(-v for v in o) for o in self.offsets])

    def RemoveCenter(self) -> "NeighborList":
        return NeighborList([o for o in self.offsets if any(o)] or [(0,) * self.rank])

    def maximum_extension(self):
        lo = tuple(min(o[i] for o in self.offsets) for i in range(self.rank))
        hi = tuple(max(o[i] for o in self.offsets) for i in range(self.rank))
        return lo, hi

    def __len__(self):
        return len(self.offsets)

    def __iter__(self):
        return iter(self.offsets)
