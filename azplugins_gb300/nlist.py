"""Neighbour list (mirror of ``hoomd.md.nlist.Cell`` as the azplugins tests use it,
``src/pytest/test_pair.py:337``): a binned full list at r_cut + buffer, with
bonded pairs excluded by default, rebuilt when a particle has moved more than
buffer / 2 since the last build."""

from __future__ import annotations


class Cell:
    """Cell-list neighbour list.

    Args:
        buffer (float): Neighbour list buffer width r_buff.
        exclusions (tuple): Topological exclusions; ``("bond",)`` (default) or ``()``.
    """

    def __init__(self, buffer=0.4, exclusions=("bond",)):
        if buffer < 0:
            raise ValueError("buffer must be non-negative")
        exclusions = tuple(exclusions)
        for e in exclusions:
            if e != "bond":
                raise ValueError(f"exclusion {e!r} is not supported (only 'bond')")
        self.buffer = float(buffer)
        self.exclusions = exclusions

    @property
    def exclude_bonds(self) -> bool:
        return "bond" in self.exclusions
