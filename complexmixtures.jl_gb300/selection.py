"""AtomSelection and the SoluteGroup / SolventGroup query types
(src/AtomSelection.jl:5-37, 48-59, 111-166, 290-372, 551-633)."""
from __future__ import annotations

import bisect
import warnings
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Union

import numpy as np


def set_nmols_natomspermol(indices: Sequence[int], nmols: int, natomspermol: int):
    """src/AtomSelection.jl:5-37."""
    natoms = len(indices)
    if natoms == 0:
        raise ValueError("Vector of atom indices is empty.")
    if nmols == 0 and natomspermol == 0:
        raise ValueError("Set nmols or natomspermol when defining a selection.")
    if nmols != 0:
        if natoms % nmols != 0:
            raise ValueError("Number of atoms in selection must be a multiple of nmols.")
        natomspermol = natoms // nmols
    else:
        if natoms % natomspermol != 0:
            raise ValueError("Number of atoms in selection must be a multiple of natomspermols.")
        nmols = natoms // natomspermol
    return nmols, natomspermol


@dataclass
class AtomSelection:
    """Atoms of the solute or solvent (src/AtomSelection.jl:48-59).

    ``indices`` are 1-based indices of the atoms in the structure file, in the
    order their coordinates are read; molecules are contiguous blocks of
    ``natomspermol`` atoms.
    """

    nmols: int
    natomspermol: int
    indices: List[int]
    custom_groups: bool = False
    group_atom_indices: List[List[int]] = field(default_factory=list)
    group_names: List[str] = field(default_factory=list)

    @staticmethod
    def from_indices(
        indices: Sequence[int],
        *,
        nmols: int = 0,
        natomspermol: int = 0,
        group_atom_indices: Optional[Sequence[Sequence[int]]] = None,
        group_names: Optional[Sequence[str]] = None,
    ) -> "AtomSelection":
        """Low-level constructor (src/AtomSelection.jl:290-372)."""
        indices = [int(i) for i in indices]
        group_atom_indices = [list(map(int, g)) for g in (group_atom_indices or [])]
        group_names = list(group_names or [])
        nmols, natomspermol = set_nmols_natomspermol(indices, nmols, natomspermol)
        custom_groups = len(group_atom_indices) > 0
        if not custom_groups and group_names and len(group_names) != natomspermol:
            raise ValueError(
                "The length of the group_names vector does not correspond to the number of atoms per molecule, "
                "but no atom groups vector was provided."
            )
        if custom_groups:
            index_set = set(indices)
            for inds in group_atom_indices:
                if inds != sorted(inds):
                    warnings.warn("Group indices are not sorted. The array will be sorted for faster search.")
                    inds.sort()
                if len(set(inds)) != len(inds):
                    raise ValueError(
                        "Found repeated indices in custom group atom indices. The group atom indices must have "
                        "unique entries."
                    )
                if any(i not in index_set for i in inds):
                    raise ValueError(
                        "Group atom indices not found in the the current AtomSelection main atomic indices."
                    )
            if not group_names:
                warnings.warn(
                    "Vector of group atom indices was provided but vector of group names is empty. The group "
                    "contributions will be only retrieved by the group indices."
                )
            elif len(group_atom_indices) != len(group_names):
                raise ValueError(
                    "The vector of group atom indices has a different number of elements than the vector of "
                    "group names."
                )
        return AtomSelection(nmols, natomspermol, indices, custom_groups, group_atom_indices, group_names)

    def natoms(self) -> int:
        return len(self.indices)

    def ngroups(self) -> int:
        return len(self.group_atom_indices) if self.custom_groups else self.natomspermol

    # ------------------------------------------------------------------ groups
    def groups_of_index(self, iat: int) -> List[int]:
        """Custom groups (0-based) that contain original atom index ``iat``:
        the searchsortedfirst lookup of src/update_counters.jl:27-33."""
        out = []
        for g, inds in enumerate(self.group_atom_indices):
            k = bisect.bisect_left(inds, iat)
            if k < len(inds) and inds[k] == iat:
                out.append(g)
        return out

    def solute_credit_table(self):
        """Per local atom of one molecule, the groups credited when that atom is
        the solute side of a minimum-distance pair, or None for default groups.

        The reference identifies the solute atom by its index inside the
        molecule (``md.i`` of CellListMap's x set) and looks it up as
        ``sol.indices[md.i]`` (src/update_counters.jl:27, :279), i.e. through the
        atoms of the selection's first molecule."""
        if not self.custom_groups:
            return None
        return [self.groups_of_index(self.indices[a]) for a in range(self.natomspermol)]

    def solvent_credit_table(self):
        """Per atom of the whole selection, the groups credited when that atom
        is the solvent side of a pair (``md.j`` is global), or None."""
        if not self.custom_groups:
            return None
        return [self.groups_of_index(i) for i in self.indices]

    def __eq__(self, other):
        if not isinstance(other, AtomSelection):
            return NotImplemented
        return (
            self.nmols == other.nmols
            and self.natomspermol == other.natomspermol
            and list(self.indices) == list(other.indices)
            and self.custom_groups == other.custom_groups
            and [list(g) for g in self.group_atom_indices] == [list(g) for g in other.group_atom_indices]
            and list(self.group_names) == list(other.group_names)
        )


def atom_group(atsel: AtomSelection, i: Union[int, str]) -> List[int]:
    """Atoms of a custom group, by 1-based index or name (src/AtomSelection.jl:111-125)."""
    if not atsel.custom_groups:
        raise ValueError("Custom groups not defined in this AtomSelection.")
    if isinstance(i, str):
        if i not in atsel.group_names:
            raise ValueError(f"Could not find group with name {i}.")
        return atsel.group_atom_indices[atsel.group_names.index(i)]
    return atsel.group_atom_indices[i - 1]


def atom_group_name(atsel: AtomSelection, i: int) -> str:
    return atsel.group_names[i - 1]


def atom_group_names(atsel: AtomSelection) -> List[str]:
    return atsel.group_names


@dataclass
class _Group:
    group_index: Optional[int] = None
    group_name: Optional[str] = None
    atom_indices: Optional[List[int]] = None
    atom_names: Optional[List[str]] = None


def _make_group(cls, arg):
    if isinstance(arg, AtomSelection):
        raise ValueError(f"No constructor for {cls.__name__} with these arguments.")
    if isinstance(arg, (bool, np.bool_)):
        raise ValueError(f"No constructor for {cls.__name__} with these arguments.")
    if isinstance(arg, (int, np.integer)):
        return cls(group_index=int(arg))
    if isinstance(arg, str):
        return cls(group_name=arg)
    seq = list(arg)
    if len(seq) == 0:
        # an empty vector: typed by its element type in the reference; the
        # contributions() error is the same for both
        return cls(atom_indices=[])
    if all(isinstance(x, str) for x in seq):
        return cls(atom_names=seq)
    if all(isinstance(x, (int, np.integer)) for x in seq):
        return cls(atom_indices=[int(x) for x in seq])
    raise ValueError(f"No constructor for {cls.__name__} with these arguments.")


class SoluteGroup(_Group):
    """Selects solute atoms for ``contributions`` (src/AtomSelection.jl:551-561, 621-626)."""

    def __init__(self, arg=None, *, group_index=None, group_name=None, atom_indices=None, atom_names=None):
        if arg is not None:
            g = _make_group(_Group, arg)
            super().__init__(g.group_index, g.group_name, g.atom_indices, g.atom_names)
        else:
            super().__init__(group_index, group_name, atom_indices, atom_names)


class SolventGroup(_Group):
    """Selects solvent atoms for ``contributions`` (src/AtomSelection.jl:563-573, 628-633)."""

    def __init__(self, arg=None, *, group_index=None, group_name=None, atom_indices=None, atom_names=None):
        if arg is not None:
            g = _make_group(_Group, arg)
            super().__init__(g.group_index, g.group_name, g.atom_indices, g.atom_names)
        else:
            super().__init__(group_index, group_name, atom_indices, atom_names)
