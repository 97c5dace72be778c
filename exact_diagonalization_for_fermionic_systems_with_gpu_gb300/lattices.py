"""Lattice term lists, matching the reference's lattice builder functions.

Each builder returns the ordered list of one-spin terms the reference applies
to one H_TBq (the same list is used for both spins, as in the reference
drivers).  A term is ``(kind, i, j, value, phase)`` with kind one of
``"H"`` (Make_H), ``"J"`` (Make_J), ``"N"`` (Make_N) or ``"P"`` (Peierls hop).
The bond tables are the reference's own (the lattices must be identical for
parity); their sources are cited per function.
"""
from __future__ import annotations

import math
from typing import List, Sequence, Tuple

Term = Tuple[str, int, int, float, float]

# DrudeWeight/src/drude_v2_cal_Kagome_randomHop.cu:796-797 (KagomeLattice12);
# identical list in TotalSpin/src/ConservedTotalSpin_Kagome_randomHop.cu:142-143
KAGOME12_FIRST = [0, 1, 3, 4, 6, 7, 9, 10, 0, 2, 6, 8, 3, 5, 9, 11, 2, 1, 8, 7, 5, 4, 11, 10]
KAGOME12_SECOND = [1, 3, 4, 0, 7, 9, 10, 6, 2, 6, 8, 0, 5, 9, 11, 3, 1, 11, 7, 5, 4, 8, 10, 2]
# x projections of the same bonds: drude_v2_cal_Kagome_randomHop.cu:818-820 (kinetic, dx^2)
# and :849-851 (current, dx)
KAGOME12_DX = [1.0] * 8 + [0.5] * 16
# y bonds and projection: drude_v2_cal_Kagome_randomHop.cu:822-828, 853-859
KAGOME12_Y_FIRST = [0, 2, 6, 8, 3, 5, 9, 11, 1, 11, 7, 5, 4, 8, 10, 2]
KAGOME12_Y_SECOND = [2, 6, 8, 0, 5, 9, 11, 3, 2, 1, 8, 7, 5, 4, 11, 10]
KAGOME12_DY = math.sqrt(3.0) / 2.0
# Linear size of the 12-site cluster along x in bond lengths (2 unit cells of
# length 2): the flux quantum of a twist is 2*pi/KAGOME12_LX per unit dx.
KAGOME12_LX = 4.0

# TotalSpin/src/TotalSpinExcited_Lieb_randomHop.cu:178-179 (LiebLattice12, bonds 3 and 7 carry +1)
LIEB12_FIRST = [0, 1, 3, 4, 6, 7, 9, 10, 0, 2, 6, 8, 3, 5, 9, 11]
LIEB12_SECOND = [1, 3, 4, 0, 7, 9, 10, 6, 2, 6, 8, 0, 5, 9, 11, 3]
# TotalSpin/src/TotalSpinExcited_Lieb_randomHop.cu:192-195 (LiebLattice18)
LIEB18_FIRST = [0, 1, 8, 9, 15, 17, 3, 4, 11, 6, 12, 14, 3, 2, 8, 7, 12, 13, 0, 5, 11, 10, 15, 16]
LIEB18_SECOND = [1, 8, 9, 15, 17, 0, 4, 11, 6, 12, 14, 3, 2, 8, 7, 12, 13, 0, 5, 11, 10, 15, 16, 3]


def chain(L: int, t: float = -1.0, periodic: bool = True, eps: Sequence[float] | None = None) -> List[Term]:
    """Nearest-neighbour chain: Make_H(i, i+1, t) for i < L-1 (the reference
    open chains Line10/Line12/Line16, MBL_test/src/Hubbard_EE_test.cu:102-140,
    use t = -1), plus Make_H(L-1, 0, t) when periodic (the Jordan-Wigner
    string of that bond makes it a true fermionic ring), plus Make_N(i, eps_i)."""
    terms: List[Term] = [("H", i, i + 1, t, 0.0) for i in range(L - 1)]
    if periodic and L > 2:
        terms.append(("H", L - 1, 0, t, 0.0))
    if eps is not None:
        terms += [("N", i, 0, float(eps[i]), 0.0) for i in range(L)]
    return terms


def kagome12(rand: Sequence[float] | None = None, onsite_shift: bool = True, flux: float = 0.0,
             peierls: bool = False) -> List[Term]:
    """KagomeLattice12 (drude_v2_cal_Kagome_randomHop.cu:794-808): hopping
    -r_i r_j on the 24 bonds and, with onsite_shift, Make_N(i, -2 r_i^2).
    With flux != 0 (or peierls=True, which keeps the operator complex at
    flux 0) every bond carries the Peierls phase flux * dx_b."""
    r = [1.0] * 12 if rand is None else list(rand)
    terms: List[Term] = []
    for b, (i, j) in enumerate(zip(KAGOME12_FIRST, KAGOME12_SECOND)):
        t = -r[i] * r[j]
        if flux != 0.0 or peierls:
            terms.append(("P", i, j, t, flux * KAGOME12_DX[b]))
        else:
            terms.append(("H", i, j, t, 0.0))
    if onsite_shift:
        terms += [("N", i, 0, -2.0 * r[i] * r[i], 0.0) for i in range(12)]
    return terms


def kagome12_kinetic_x(rand: Sequence[float] | None = None) -> List[Term]:
    """KagomeKinetic12 x part (drude_v2_cal_Kagome_randomHop.cu:830-833):
    Make_H(i, j, -r_i r_j dx^2)."""
    r = [1.0] * 12 if rand is None else list(rand)
    return [("H", i, j, -r[i] * r[j] * KAGOME12_DX[b] ** 2, 0.0)
            for b, (i, j) in enumerate(zip(KAGOME12_FIRST, KAGOME12_SECOND))]


def kagome12_current_x(rand: Sequence[float] | None = None) -> List[Term]:
    """KagomeCurrent12 x part (drude_v2_cal_Kagome_randomHop.cu:861-864):
    Make_J(i, j, r_i r_j dx)."""
    r = [1.0] * 12 if rand is None else list(rand)
    return [("J", i, j, r[i] * r[j] * KAGOME12_DX[b], 0.0)
            for b, (i, j) in enumerate(zip(KAGOME12_FIRST, KAGOME12_SECOND))]


def kagome12_kinetic_y(rand: Sequence[float] | None = None) -> List[Term]:
    r = [1.0] * 12 if rand is None else list(rand)
    return [("H", i, j, -r[i] * r[j] * 0.75, 0.0) for i, j in zip(KAGOME12_Y_FIRST, KAGOME12_Y_SECOND)]


def kagome12_current_y(rand: Sequence[float] | None = None) -> List[Term]:
    r = [1.0] * 12 if rand is None else list(rand)
    return [("J", i, j, r[i] * r[j] * KAGOME12_DY, 0.0) for i, j in zip(KAGOME12_Y_FIRST, KAGOME12_Y_SECOND)]


def lieb12(rand: Sequence[float] | None = None) -> List[Term]:
    """LiebLattice12 (TotalSpinExcited_Lieb_randomHop.cu:176-188)."""
    r = [1.0] * 12 if rand is None else list(rand)
    out: List[Term] = []
    for b, (i, j) in enumerate(zip(LIEB12_FIRST, LIEB12_SECOND)):
        p = 1.0 if b in (3, 7) else -1.0
        out.append(("H", i, j, p * r[i] * r[j], 0.0))
    return out


def lieb18(rand: Sequence[float] | None = None) -> List[Term]:
    """LiebLattice18 (TotalSpinExcited_Lieb_randomHop.cu:190-202)."""
    r = [1.0] * 18 if rand is None else list(rand)
    return [("H", i, j, -r[i] * r[j], 0.0) for i, j in zip(LIEB18_FIRST, LIEB18_SECOND)]


def squared_3by4(t: float = -1.0) -> List[Term]:
    """Squared_3by4 (MBL_test/src/Hubbard_test.cu:126-157), open 3x4 square lattice."""
    bonds = [(0, 1), (1, 2), (2, 3), (4, 5), (5, 6), (6, 7), (8, 9), (9, 10), (10, 11),
             (0, 4), (4, 8), (1, 5), (5, 9), (2, 6), (6, 10), (3, 7), (7, 11)]
    return [("H", i, j, t, 0.0) for i, j in bonds]


def kagome12_flux_derivatives(flux: float, rand: Sequence[float] | None = None):
    """d/dPhi and d^2/dPhi^2 of the twisted Kagome12 hopping: with bond phase
    Phi*dx_b, dH/dPhi carries t_b dx_b e^{i(Phi dx_b + pi/2)} and d2H/dPhi2
    t_b dx_b^2 e^{i(Phi dx_b + pi)} on every bond (the on-site term does not
    depend on Phi).  At Phi = 0, d2H/dPhi2 = -K_x (KagomeKinetic12) and
    dH/dPhi = -i J_x (KagomeCurrent12)."""
    r = [1.0] * 12 if rand is None else list(rand)
    d1, d2 = [], []
    for b, (i, j) in enumerate(zip(KAGOME12_FIRST, KAGOME12_SECOND)):
        t = -r[i] * r[j]
        dx = KAGOME12_DX[b]
        d1.append(("P", i, j, t * dx, flux * dx + math.pi / 2))
        d2.append(("P", i, j, t * dx * dx, flux * dx + math.pi))
    return d1, d2


def hopping_only(terms: List[Term]) -> List[Term]:
    """The kinetic part of a term list (drops Make_N terms)."""
    return [t for t in terms if t[0] != "N"]
