"""Group contribution queries on a finished Result
(src/tools/contributions.jl:70-248, src/tools/coordination_number.jl:104-106).
Pure host post-processing of the group counters the engine produced."""
from __future__ import annotations

import numpy as np

from .results import Result, _jcumsum, units
from .selection import SoluteGroup, SolventGroup


def _summary(x) -> str:
    x = list(x)
    if len(x) <= 4:
        return "[ " + ", ".join(map(str, x)) + " ]"
    return "[ " + ", ".join(map(str, x[:2])) + ", ..., " + ", ".join(map(str, x[-2:])) + " ]"


def contributions(R: Result, group, *, type: str = "mddf", _warn_zero_md_count: bool = True) -> np.ndarray:
    """Contribution of a solute or solvent group to the MDDF (``type="mddf"``),
    coordination number, md count or KB integral (src/tools/contributions.jl:70-248)."""
    if type not in ("mddf", "coordination_number", "md_count", "kbi"):
        raise ValueError("type must be :mddf (default), :coordination_number, :md_count, :kbi")
    if isinstance(group, SoluteGroup):
        atsel, gc, gcr = R.solute, R.solute_group_count, R.solute_group_count_random
    elif isinstance(group, SolventGroup):
        atsel, gc, gcr = R.solvent, R.solvent_group_count, R.solvent_group_count_random
    else:
        raise ValueError("group must be a SoluteGroup or SolventGroup")
    if atsel.custom_groups:
        if group.group_index is None and group.group_name is None:
            raise ValueError(
                "Custom groups are defined. Cannot retrieve general group contributions. Please provide a group "
                f"name or index. Group (or atom) names available: {_summary(atsel.group_names)}"
            )
    else:
        if group.atom_indices is None and group.atom_names is None:
            raise ValueError(
                f'The "{group.group_name}" string identifier of the group was set, but no custom group names were '
                f'defined. Please provide vectors of *atomic* indices or names. ... replace "{group.group_name}" by '
                f'select(atoms, "{group.group_name}") ?'
            )
    nb = gc.shape[1]
    sel = np.zeros(nb)
    selr = np.zeros(nb)
    if group.group_index is not None:
        ig = group.group_index
        if ig > gc.shape[0] or ig < 1:
            raise ValueError(f"Group {ig} greater than number of groups ({gc.shape[0]}) of group contribution array.")
        sel[:] = gc[ig - 1]
        selr[:] = gcr[ig - 1]
    if group.group_name is not None:
        if group.group_name not in atsel.group_names:
            raise ValueError(f'Atom (or group) name "{group.group_name}" not found in atom selection. '
                             f"Group names list: {_summary(atsel.group_names)}.")
        ig = atsel.group_names.index(group.group_name)
        sel[:] = gc[ig]
        selr[:] = gcr[ig]
    if group.atom_indices is not None:
        if len(group.atom_indices) == 0:
            raise ValueError("Group selection by group indices is empty.")
        if len(set(group.atom_indices)) != len(group.atom_indices):
            raise ValueError("Selection by atom indices contains repeated indices.")
        pos = {idx: k for k, idx in enumerate(atsel.indices)}
        if atsel.nmols == 1:
            for iat in group.atom_indices:
                if iat not in pos:
                    raise ValueError(f"Atom index {iat} not found in atom selection. Indices array: {_summary(atsel.indices)}.")
                sel += gc[pos[iat]]
                selr += gcr[pos[iat]]
        else:
            first = atsel.indices[0]
            for iat in group.atom_indices:
                if iat not in pos:
                    raise ValueError(f"Atom index {iat} not found in atom selection. Indices array: {_summary(atsel.indices)}.")
                itype = (iat - first) % atsel.natomspermol  # atom_type(iat, n; first) - 1
                sel += gc[itype] / atsel.nmols
                selr += gcr[itype] / atsel.nmols
    if group.atom_names is not None:
        if len(group.atom_names) == 0:
            raise ValueError("Selection by atom names is empty.")
        if len(set(group.atom_names)) != len(group.atom_names):
            raise ValueError("Selection by atom names contains repeated names.")
        for name in group.atom_names:
            found = False
            for ig, gname in enumerate(atsel.group_names):
                if gname == name:
                    found = True
                    sel += gc[ig]
                    selr += gcr[ig]
            if not found:
                raise ValueError(f'Atom (or group) name "{name}" not found in atom selection. '
                                 f"Group names list: {_summary(atsel.group_names)}.")
    if type == "mddf":
        out = np.zeros(nb)
        for i in range(nb):
            out[i] = 0.0 if R.md_count_random[i] == 0.0 else sel[i] / R.md_count_random[i]
        return out
    if type == "coordination_number":
        return _jcumsum(sel)
    if type == "md_count":
        return sel
    return units.Angs3tocm3permol * (1 / R.density.solvent_bulk) * (_jcumsum(sel) - _jcumsum(selr))


def coordination_number(R: Result, group=None) -> np.ndarray:
    """R.coordination_number, or the group's cumulative contribution
    (src/tools/coordination_number.jl:104-106)."""
    if group is None:
        return R.coordination_number
    return contributions(R, group, type="coordination_number")
