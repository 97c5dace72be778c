"""The reference drivers' file formats, so runs of this library slot into the
same analysis scripts.

Disorder files  `<path>/randNum_<Lattice>-L<N>.dat`
    written by TotalSpin/src/randNum_generator.cpp:30-51: a header line
    "#       X_1        X_2     ....    " when the file is new (appended to
    otherwise), then one line per sample, N numbers each followed by a tab,
    printed by an ostream with precision(10);
    read by TotalSpinExcited_Lieb_randomHop.cu:90-127: lines starting with '#'
    are skipped, N numbers per line, site factor r_i = 1 + X * number.

Result files  e.g. DrudeWeight_v2_Kagome-L<N>aU<U>Q<Q>X<X>.dat
    drude_v2_cal_Kagome_randomHop.cu:112-124,157-158: a '#' header line when
    the file is new (append mode otherwise), precision(10), each data row a
    tab before every value, newline at the end.

Numbers are formatted as C++ ostream's default floating-point notation with
precision 10, i.e. printf's "%.10g".  Random numbers come from
Philox4x64-10 (seed, sample) instead of the reference's std::mt19937 seeded
from std::random_device (which cannot be reproduced).
"""
from __future__ import annotations

import os
from typing import Iterable, List, Sequence

import numpy as np

from .hubbard import random_vector

RANDNUM_HEADER = "#       X_1        X_2     ....    "


def fmt10(v: float) -> str:
    """A double as `std::ostream << v` with precision(10) prints it."""
    return "%.10g" % float(v)


def randnum_filename(path: str, lattice: str, n_sites: int) -> str:
    return os.path.join(path, f"randNum_{lattice}-L{n_sites}.dat")


def random_numbers(n_samples: int, n_sites: int, seed: int = 0) -> np.ndarray:
    """uniform(-1, 1) disorder numbers, sample s from Philox4x64-10 keyed by
    seed * 2^20 + s (n_samples x n_sites)."""
    if n_samples == 0:
        return np.zeros((0, n_sites))
    return np.stack([random_vector(n_sites, seed * (1 << 20) + s) for s in range(n_samples)])


def write_random_numbers(path: str, lattice: str, samples: np.ndarray) -> str:
    """Append samples (n_samples x N) to randNum_<lattice>-L<N>.dat, creating it
    with the reference header when it does not exist.  Returns the file name."""
    samples = np.atleast_2d(np.asarray(samples, dtype=np.float64))
    fn = randnum_filename(path, lattice, samples.shape[1])
    new = not os.path.exists(fn)
    with open(fn, "a") as f:
        if new:
            f.write(RANDNUM_HEADER + "\n")
        for row in samples:
            f.write("".join(fmt10(v) + "\t" for v in row) + "\n")
    return fn


def read_random_numbers(path: str, lattice: str, n_sites: int) -> np.ndarray:
    """All samples of randNum_<lattice>-L<N>.dat ('#' lines skipped; N numbers
    per line, extra fields ignored as the reference's istringstream does)."""
    fn = randnum_filename(path, lattice, n_sites)
    rows: List[List[float]] = []
    with open(fn) as f:
        for line in f:
            if line.startswith("#") or not line.strip():
                continue
            vals = line.split()
            if len(vals) < n_sites:
                raise ValueError(f"{fn}: a sample line has {len(vals)} numbers, {n_sites} expected")
            rows.append([float(v) for v in vals[:n_sites]])
    return np.array(rows).reshape(len(rows), n_sites)


def site_factors(numbers: Sequence[float], X: float) -> np.ndarray:
    """r_i = 1 + X * number_i (TotalSpinExcited_Lieb_randomHop.cu:117)."""
    return 1.0 + X * np.asarray(numbers, dtype=np.float64)


def append_rows(filename: str, header: str, rows: Iterable[Sequence[float]]) -> None:
    """Append data rows ("\\t" before each value, precision 10) to a result
    file, writing `header` first when the file is new."""
    new = not os.path.exists(filename)
    with open(filename, "a") as f:
        if new:
            f.write(header + "\n")
        for r in rows:
            f.write("".join("\t" + fmt10(v) for v in r) + "\n")


def drude_filename(path: str, n_sites: int, U: str, Q: str, X: str) -> str:
    """DrudeWeight_v2_Kagome-L<N>aU<U>Q<Q>X<X>.dat (drude_v2_cal_Kagome_randomHop.cu:112-114);
    U, Q, X as the strings the driver was given on its command line."""
    return os.path.join(path, f"DrudeWeight_v2_Kagome-L{n_sites}aU{U}Q{Q}X{X}.dat")


DRUDE_HEADER = "#       E       Dxx        Dyy        D      "
