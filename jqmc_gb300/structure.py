"""Nuclear structure and the nearest-nucleus helpers used on the walker path.

Mirrors ``jqmc/structure.py``: ``Structure_data`` (structure.py:66) and the
nearest-nucleus search ``_find_nearest_nucleus_indices_np`` (structure.py:393-405),
``_get_min_dist_rel_R_cart_np`` (structure.py:428-453).  Periodic boundary
conditions are not supported on this path (``pbc_flag`` must be False).
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass(frozen=True)
class Structure_data:
    """Nuclear positions (bohr) and labels; see jqmc/structure.py:66."""

    positions: np.ndarray = field(default_factory=lambda: np.zeros((0, 3)))
    pbc_flag: bool = False
    atomic_numbers: tuple = ()
    element_symbols: tuple = ()
    atomic_labels: tuple = ()

    def __post_init__(self):
        object.__setattr__(self, "positions", np.asarray(self.positions, dtype=np.float64).reshape(-1, 3))

    @property
    def natom(self) -> int:
        return int(self.positions.shape[0])

    @property
    def _positions_cart_np(self) -> np.ndarray:
        return self.positions

    def sanity_check(self) -> None:
        if self.pbc_flag:
            raise NotImplementedError("periodic systems are not supported on the walker path")
        if len(self.atomic_numbers) != self.natom:
            raise ValueError(f"len(atomic_numbers)={len(self.atomic_numbers)} != natom={self.natom}")


def find_nearest_index(structure: Structure_data, r_cart) -> int:
    """Index of the nucleus nearest to ``r_cart`` (ties resolve to the lower index,
    as the stable argsort of structure.py:393-405 does)."""
    d = np.sqrt(np.sum((structure.positions - np.asarray(r_cart)) ** 2, axis=1))
    return int(np.argsort(d, kind="stable")[0])
