"""Group contribution queries on a finished Result
(src/tools/contributions.jl:70-248, src/tools/coordination_number.jl:104-106).
Pure host post-processing of the group counters the engine produced."""
from __future__ import annotations

import numpy as np

from .results import Result, _jcumsum, sum_frame_weights, units
from .selection import SoluteGroup, SolventGroup


def _summary(x) -> str:
    x = list(x)
    if len(x) <= 4:
        return "[ " + ", ".join(map(str, x)) + " ]"
    return "[ " + ", ".join(map(str, x[:2])) + ", ..., " + ", ".join(map(str, x[-2:])) + " ]"


CONTRIB_TYPES = ("mddf", "coordination_number", "md_count", "kbi")


def contribution_terms(R: Result, group):
    """Resolve a SoluteGroup / SolventGroup into the reference's summation:
    (side, rows, divide), where ``rows`` are the 0-based group rows added to
    sel_count in the reference's order and ``divide`` says whether each is
    divided by the selection's nmols (atom indices of a multi-molecule
    selection).  Raises the reference's argument errors
    (src/tools/contributions.jl:102-215)."""
    if isinstance(group, SoluteGroup):
        side, atsel, ng = "solute", R.solute, R.solute_group_count.shape[0]
    elif isinstance(group, SolventGroup):
        side, atsel, ng = "solvent", R.solvent, R.solvent_group_count.shape[0]
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
    # sel_count .= group_count[ig] on a zero vector is the sum of that one row
    rows = []
    divide = False
    if group.group_index is not None:
        ig = group.group_index
        if ig > ng or ig < 1:
            raise ValueError(f"Group {ig} greater than number of groups ({ng}) of group contribution array.")
        rows = [ig - 1]
    if group.group_name is not None:
        if group.group_name not in atsel.group_names:
            raise ValueError(f'Atom (or group) name "{group.group_name}" not found in atom selection. '
                             f"Group names list: {_summary(atsel.group_names)}.")
        rows = [atsel.group_names.index(group.group_name)]
    if group.atom_indices is not None:
        if len(group.atom_indices) == 0:
            raise ValueError("Group selection by group indices is empty.")
        if len(set(group.atom_indices)) != len(group.atom_indices):
            raise ValueError("Selection by atom indices contains repeated indices.")
        pos = {idx: k for k, idx in enumerate(atsel.indices)}
        for iat in group.atom_indices:
            if iat not in pos:
                raise ValueError(f"Atom index {iat} not found in atom selection. Indices array: {_summary(atsel.indices)}.")
        if atsel.nmols == 1:
            rows += [pos[iat] for iat in group.atom_indices]
        else:
            first = atsel.indices[0]
            rows += [(iat - first) % atsel.natomspermol for iat in group.atom_indices]  # atom_type(iat, n; first) - 1
            divide = True
    if group.atom_names is not None:
        if len(group.atom_names) == 0:
            raise ValueError("Selection by atom names is empty.")
        if len(set(group.atom_names)) != len(group.atom_names):
            raise ValueError("Selection by atom names contains repeated names.")
        for name in group.atom_names:
            found = [ig for ig, gname in enumerate(atsel.group_names) if gname == name]
            if not found:
                raise ValueError(f'Atom (or group) name "{name}" not found in atom selection. '
                                 f"Group names list: {_summary(atsel.group_names)}.")
            rows += found
    return side, rows, divide, atsel.nmols


def _check_type(type: str) -> None:
    if type not in CONTRIB_TYPES:
        raise ValueError("type must be :mddf (default), :coordination_number, :md_count, :kbi")


def _warn_zero_random(R: Result, type: str, warn: bool) -> None:
    if warn and type == "mddf" and np.all(R.md_count_random == 0):
        import warnings

        warnings.warn("This is probably a `coordination_number` calculation only. To compute the contributions to "
                      "coordination numbers, use `type=:coordination_number`.")


def _engine_of(R: Result, engine):
    return engine if engine is not None else getattr(R, "engine", None)


def contributions(R: Result, group, *, type: str = "mddf", _warn_zero_md_count: bool = True, engine=None) -> np.ndarray:
    """Contribution of a solute or solvent group to the MDDF (``type="mddf"``),
    coordination number, md count or KB integral (src/tools/contributions.jl:70-248).

    With an open ``engine`` holding the run's accumulators (the ``engine``
    argument, or ``R.engine`` left by ``mddf(..., keep_engine=True)``) the sum
    and conversion run on the GPU (cm_contributions); otherwise on the host.
    Both follow the reference's order of FP64 operations."""
    _check_type(type)
    side, rows, divide, nmols = contribution_terms(R, group)
    _warn_zero_random(R, type, _warn_zero_md_count)
    eng = _engine_of(R, engine)
    if eng is not None:
        return eng.contributions([(side, type, rows, divide)], sum_frame_weights(R))[0]
    gc, gcr = ((R.solute_group_count, R.solute_group_count_random) if side == "solute"
               else (R.solvent_group_count, R.solvent_group_count_random))
    nb = gc.shape[1]
    sel = np.zeros(nb)
    selr = np.zeros(nb)
    for g in rows:
        sel += gc[g] / nmols if divide else gc[g]
        selr += gcr[g] / nmols if divide else gcr[g]
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


def _residues(atoms):
    """Consecutive runs of atoms of one residue (PDBTools.eachresidue): same
    residue number, name and chain."""
    out = []
    for k in range(len(atoms.xyz)):
        key = (atoms.resnum[k], atoms.resname[k], atoms.chain[k])
        if out and out[-1][0] == key:
            out[-1][1].append(k)
        else:
            out.append((key, [k]))
    return out


class ResidueContributions:
    """Contributions of each residue of the solute to the MDDF (or
    coordination number, md count, KBI) between dmin and dmax
    (src/tools/residue_contributions.jl:157-215), with the reference's
    slicing, iteration and arithmetic (src/tools/residue_contributions.jl:239-373).

    ``ResidueContributions(results, atoms, dmin=1.5, dmax=3.5, type="mddf")``
    with ``atoms`` an ``Atoms`` object (the solute, or part of it; atom
    indices in ``atoms.index``).  With an engine (argument, or ``R.engine``)
    all residues are one cm_contributions call: one query per residue.
    ``xticks`` are (residue numbers, residue name + number labels)."""

    def __init__(self, results: Result = None, atoms=None, *, dmin: float = 1.5, dmax: float = 3.5,
                 type: str = "mddf", silent: bool = False, engine=None, _parts=None):
        if _parts is not None:
            self.d, self.residue_contributions, self.resnums, self.xticks, self.single = _parts
            return
        if atoms is None or len(atoms.xyz) == 0:
            raise ValueError("The atom selection provided is empty.")
        if results.solute.custom_groups:
            raise ValueError("The call to ResidueContributions with a SoluteGroup or SolventGroup objects as arguments "
                             "is not valid. You must provide *the atoms* of the solute as the second argument of the "
                             "function, and the solute must have been defined without custom groups.")
        _check_type(type)
        residues = _residues(atoms)
        groups = [SoluteGroup([int(atoms.index[k]) for k in ks]) for _, ks in residues]
        eng = _engine_of(results, engine)
        if eng is not None:
            queries = []
            for g in groups:
                side, rows, divide, _ = contribution_terms(results, g)
                queries.append((side, type, rows, divide))
            _warn_zero_random(results, type, not silent)
            curves = list(eng.contributions(queries, sum_frame_weights(results)))
        else:
            curves = [contributions(results, g, type=type, _warn_zero_md_count=(not silent and i == 0))
                      for i, g in enumerate(groups)]
        d = np.asarray(results.d)
        above_min = np.nonzero(d > dmin)[0]
        above_max = np.nonzero(d > dmax)[0]
        i0 = int(above_min[0]) if len(above_min) else 0
        i1 = int(above_max[0]) if len(above_max) else len(d) - 1
        self.d = d[i0:i1 + 1].copy()
        self.residue_contributions = [np.asarray(c)[i0:i1 + 1].copy() for c in curves]
        self.resnums = [key[0] for key, _ in residues]
        self.xticks = (list(self.resnums), [f"{key[1]}{key[0]}" for key, _ in residues])
        self.single = len(residues) == 1

    def to_json(self) -> dict:
        """The reference's JSON fields of a ResidueContributions."""
        from .results import CURRENT_VERSION

        return {"Version": ".".join(map(str, CURRENT_VERSION)), "d": [float(x) for x in self.d],
                "residue_contributions": [[float(x) for x in c] for c in self.residue_contributions],
                "resnums": [int(r) for r in self.resnums],
                "xticks": [[int(x) for x in self.xticks[0]], [str(x) for x in self.xticks[1]]]}

    @classmethod
    def from_json(cls, D: dict) -> "ResidueContributions":
        """Read back to_json's fields; one residue reads as a single-residue
        object, as in the reference."""
        curves = [np.asarray(c, dtype=np.float64) for c in D["residue_contributions"]]
        if not curves:
            raise ValueError("no residue contributions")
        return cls(_parts=(np.asarray(D["d"], dtype=np.float64), curves, [int(r) for r in D["resnums"]],
                           ([int(x) for x in D["xticks"][0]], [str(x) for x in D["xticks"][1]]), len(curves) == 1))

    def _new(self, curves, resnums=None, xticks=None, single=None):
        return ResidueContributions(_parts=(self.d.copy(), curves, list(self.resnums if resnums is None else resnums),
                                            (list((xticks or self.xticks)[0]), list((xticks or self.xticks)[1])),
                                            self.single if single is None else single))

    def copy(self):
        return self._new([c.copy() for c in self.residue_contributions])

    def __len__(self):
        return len(self.residue_contributions[0]) if self.single else len(self.residue_contributions)

    def __getitem__(self, r):
        if self.single:
            return self.residue_contributions[0][r]
        if isinstance(r, (int, np.integer)):
            r = slice(int(r), int(r) + 1 if r != -1 else None)
        idx = list(range(len(self.residue_contributions)))[r]
        return self._new([self.residue_contributions[i] for i in idx], [self.resnums[i] for i in idx],
                         ([self.xticks[0][i] for i in idx], [self.xticks[1][i] for i in idx]), len(idx) == 1)

    def __iter__(self):
        if self.single:
            return iter(self.residue_contributions[0])
        return (self[i] for i in range(len(self.residue_contributions)))

    def __eq__(self, other):
        return (isinstance(other, ResidueContributions) and np.array_equal(self.d, other.d)
                and self.xticks == other.xticks and self.resnums == other.resnums
                and len(self.residue_contributions) == len(other.residue_contributions)
                and all(np.array_equal(a, b) for a, b in zip(self.residue_contributions, other.residue_contributions)))

    def _check(self, other):
        if not np.array_equal(self.d, other.d):
            raise ValueError("Cannot operate on these contributions: the distance vectors in the two "
                             "ResidueContributions objects differ.")
        if len(self.residue_contributions) != len(other.residue_contributions):
            raise ValueError("Cannot operate on these contributions: the number of residues in the two "
                             "ResidueContributions objects differ.")
        if self.xticks[1] != other.xticks[1]:
            import warnings

            warnings.warn("The residue tick labels in the two ResidueContributions objects differ. The resulting "
                          "tick labels will be from the first object.")

    def _binary(self, other, op):
        if isinstance(other, ResidueContributions):
            self._check(other)
            return self._new([op(a, b) for a, b in zip(self.residue_contributions, other.residue_contributions)])
        return NotImplemented

    def __add__(self, other):
        return self._binary(other, lambda a, b: a + b)

    def __sub__(self, other):
        return self._binary(other, lambda a, b: a - b)

    def __mul__(self, other):
        if isinstance(other, ResidueContributions):
            return self._binary(other, lambda a, b: a * b)
        return self._new([c * float(other) for c in self.residue_contributions])

    __rmul__ = __mul__

    def __truediv__(self, other):
        if isinstance(other, ResidueContributions):
            if any(np.any(c == 0) for c in other.residue_contributions):
                import warnings

                warnings.warn("Division by zero detected. These elements will be set to zero.")
            return self._binary(other, lambda a, b: np.where(b == 0, 0.0, a / np.where(b == 0, 1.0, b)))
        return self * (1.0 / float(other))


def coordination_number(R: Result, group=None) -> np.ndarray:
    """R.coordination_number, or the group's cumulative contribution
    (src/tools/coordination_number.jl:104-106)."""
    if group is None:
        return R.coordination_number
    return contributions(R, group, type="coordination_number")
