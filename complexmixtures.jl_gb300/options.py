"""Options: the input parameters of an MDDF run (src/Options.jl:6-192)."""
from __future__ import annotations

import warnings
from dataclasses import dataclass, field
from typing import List, Optional, Sequence


@dataclass(frozen=True)
class Options:
    """Immutable run options with the validation of the reference's keyword
    constructor (src/Options.jl:68-192).  Build with :func:`make_options` or
    ``Options.create(...)``; the dataclass fields are the reference's fields."""

    firstframe: int = 1
    lastframe: int = -1
    stride: int = 1
    irefatom: int = -1
    n_random_samples: int = 10
    binstep: float = 0.02
    dbulk: float = 10.0
    cutoff: float = 10.0
    usecutoff: bool = False
    lcell: int = 1
    GC: bool = True
    GC_threshold: float = 0.3
    seed: int = 321
    StableRNG: bool = False
    nthreads: int = 0
    silent: bool = False

    @staticmethod
    def create(**kw) -> "Options":
        return make_options(**kw)


def make_options(
    *,
    firstframe: int = 1,
    lastframe: int = -1,
    stride: int = 1,
    irefatom: int = -1,
    n_random_samples: int = 10,
    binstep: float = 0.02,
    dbulk: Optional[float] = None,
    cutoff: Optional[float] = None,
    usecutoff: Optional[bool] = None,
    bulk_range: Optional[Sequence[float]] = None,
    lcell: int = 1,
    GC: bool = True,
    GC_threshold: float = 0.3,
    seed: int = 321,
    StableRNG: bool = False,
    nthreads: int = 0,
    silent: bool = False,
) -> Options:
    """Keyword constructor restating src/Options.jl:68-192 (same defaults,
    same ArgumentError cases, raised here as ValueError)."""
    warn = False
    if stride < 1:
        raise ValueError("in MDDF options: stride cannot be less than 1. ")
    if lastframe > 0 and lastframe < firstframe:
        raise ValueError("in MDDF options: lastframe must be greater or equal to firstframe. ")
    if n_random_samples < 1:
        raise ValueError(
            "in MDDF options: n_random_samples must be greater than 0. To skip the normalization of the "
            "distribution, use the coordination_number(...) function instead of mddf(...)."
        )
    if bulk_range is not None and any(x is not None for x in (dbulk, cutoff, usecutoff)):
        raise ValueError("The bulk_range argument implies that dbulk, cutoff, and usecutoff are not needed. ")
    if all(x is None for x in (bulk_range, dbulk, cutoff, usecutoff)):
        dbulk, cutoff, usecutoff = 10.0, 10.0, False
        warn = True
    elif bulk_range is not None:
        if len(bulk_range) != 2:
            raise ValueError(
                "bulk_range must be a tuple or vector with two elements, corresponding to dbulk and cutoff."
            )
        dbulk, cutoff = bulk_range
        usecutoff = True
    else:
        if dbulk is None:
            dbulk = 10.0
            warn = True
        if usecutoff is None:
            usecutoff = False
            warn = True
        if cutoff is None:
            warn = True
            cutoff = dbulk + 4.0 if usecutoff else dbulk
        elif not usecutoff:
            raise ValueError("in MDDF options: cutoff was defined with usecutoff set to false")
    dbulk = float(dbulk)
    cutoff = float(cutoff)
    if warn and not silent:
        warnings.warn(
            f"Using default values for dbulk, cutoff and/or usecutoff: dbulk = {dbulk}, cutoff = {cutoff}, "
            f"usecutoff = {usecutoff}.  It is recommended to set bulk_range manually.",
            stacklevel=2,
        )
    if usecutoff and dbulk >= cutoff:
        raise ValueError(" in MDDF options: The bulk volume is zero (dbulk must be smaller than cutoff). ")
    # Julia's % on floats is rem (sign of the dividend)
    if _rem1(cutoff / binstep) > 1.0e-5:
        raise ValueError("in MDDF options: cutoff must be a multiple of binstep.")
    if _rem1(dbulk / binstep) > 1.0e-5:
        raise ValueError("in MDDF options: dbulk must be a multiple of binstep.")
    return Options(
        firstframe=firstframe,
        lastframe=lastframe,
        stride=stride,
        irefatom=irefatom,
        n_random_samples=n_random_samples,
        binstep=float(binstep),
        dbulk=dbulk,
        cutoff=cutoff,
        usecutoff=bool(usecutoff),
        lcell=lcell,
        GC=GC,
        GC_threshold=GC_threshold,
        seed=seed,
        StableRNG=StableRNG,
        nthreads=nthreads,
        silent=silent,
    )


def _rem1(x: float) -> float:
    import math

    return math.fmod(x, 1.0)


@dataclass
class TrajectoryFileOptions:
    """Per-file metadata kept in a Result (src/Options.jl:274-283)."""

    filename: str
    options: Options
    irefatom: int
    lastframe_read: int
    nframes_read: int
    frame_weights: List[float] = field(default_factory=list)
