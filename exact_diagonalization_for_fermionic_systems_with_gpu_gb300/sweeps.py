"""Parameter sweeps of the reference drivers, run through this library's
ground-state path on one GPU.

flux_sweep   Kagome12 6+6 with a twist Phi on every bond (phase Phi * dx_b):
             E0, dE0/dPhi (Hellmann-Feynman) and d2E0/dPhi2 (linear response)
             at n_phi points of [0, 2 pi / KAGOME12_LX].  d2E0/dPhi2 at
             Phi = 0 is the twist-curvature form of the Drude weight that
             DrudeWeight/src/drude_v2_cal_Kagome_randomHop.cu:144-155 obtains
             from <K_x> and the current-current Kubo sum (drude_weight_Jx).
mbl_sweep    open L=12 chain, t=1, U, on-site disorder W * uniform(-1, 1)
             drawn separately for the up and the down spin operator, as
             MBL_test/src/Hubbard_EE_test.cu:66-70 does with two Line16
             calls on one random stream; for every realisation and every
             (N_up, N_dn) sector: E0, the entanglement entropy of sites
             0..L/2-1 (EEmatHubAB_GPU::Make_Write + cusolverZsvd + the
             -sum S log S of Hubbard_EE_test.cu:76-83, taken here on the
             ground state instead of the reference's dense-ED quench) and
             dE0/d eps_{i,s} = <n_{i,s}> (Hellmann-Feynman on the site term).

Disorder numbers come from Philox4x64-10 keyed by (seed, realisation), so the
same realisation is used in every sector; each instance's Lanczos start
vector is keyed by realisation * n_sectors + sector.  Every quantity stays on
the device between the Lanczos run and the observables (the Ritz vector is
written into a CUDA tensor).

`python -m exact_diagonalization_for_fermionic_systems_with_gpu_gb300.sweeps
--what flux|mbl` runs a sweep and prints one JSON line with its timing.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import time
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import lattices as L
from . import observables as ob
from .hubbard import H_TBq, Hubbard, Lanczos, lanczos_batch, lanczos_multi, random_vector


@dataclass
class FluxPoint:
    phi: float
    e0: float
    d1: float          # dE0/dPhi
    d2: float          # d2E0/dPhi2
    steps: int         # Lanczos steps of the ground-state run
    min_bits: int = 0  # fewest significant bits a Lanczos vector kept (fixed-point solver)
    err_vs_oracle: float = float("nan")  # |E0 - E0 of the FP64 oracle|, where one is given


@dataclass
class MblPoint:
    realisation: int
    sector: Tuple[int, int]
    e0: float
    s_vn: float        # -sum lambda log lambda of the reduced density matrix
    s_ref: float       # the reference's -sum S log S over singular values
    n_up: np.ndarray   # dE0/d eps_{i,up}
    n_dn: np.ndarray   # dE0/d eps_{i,dn}
    steps: int
    min_bits: int = 0
    err_vs_oracle: float = float("nan")


@dataclass
class SweepTiming:
    instances: int = 0
    lanczos_steps: int = 0
    build_s: float = 0.0       # operator construction (tables, plans, upload)
    lanczos_s: float = 0.0     # ground state and Ritz vector
    observables_s: float = 0.0
    total_s: float = 0.0
    per_instance: List[float] = field(default_factory=list)

    def summary(self) -> dict:
        return {"instances": self.instances, "lanczos_steps": self.lanczos_steps,
                "total_s": round(self.total_s, 4), "build_s": round(self.build_s, 4),
                "lanczos_s": round(self.lanczos_s, 4), "observables_s": round(self.observables_s, 4),
                "instances_per_s": round(self.instances / self.total_s, 3) if self.total_s > 0 else None,
                "lanczos_steps_per_s": round(self.lanczos_steps / self.lanczos_s, 1) if self.lanczos_s > 0 else None}


def _sync():
    import torch
    if torch.cuda.is_available():
        torch.cuda.synchronize()


def _ground(H: Hubbard, steps: int, mode: str, seed: int):
    """(E0, Ritz vector as a CUDA tensor, steps taken, min_bits)."""
    import torch
    dt = torch.complex128 if H.is_complex else torch.float64
    evec = torch.empty(H.rows(), dtype=dt, device="cuda")
    lz = Lanczos()
    e0, _ = lz.eigen(H, max_steps=steps, mode=mode, ritz="stored", seed=seed, evec_out=evec)
    return e0, evec, int(lz.result.steps), int(lz.result.min_bits)


# Lanczos steps of a twist's ground state (fixed) and of its response solve.
# The twisted Kagome12 ground level comes within 0.014 of the next one
# (near Phi = 0.73, the pair split from the zero-twist doublet); the
# second-order response needs the ground state to about 1e-9 there, which
# 300 steps do not give and 500 do.
FLUX_STEPS = 500
FLUX_RESPONSE_STEPS = 200


def _real_twist(phi: float) -> bool:
    """Every bond phase phi * dx_b is a multiple of pi: the operator is real
    and time-reversal symmetric, where the ground level can be degenerate."""
    return all(abs(math.sin(phi * dx)) < 1e-15 for dx in L.KAGOME12_DX)


def flux_phis(n_phi: int = 16) -> np.ndarray:
    """n_phi twists evenly spaced over [0, 2 pi / KAGOME12_LX], both ends included."""
    return np.linspace(0.0, 2.0 * math.pi / L.KAGOME12_LX, n_phi)


def flux_sweep(phis: Optional[Sequence[float]] = None, n_up: int = 6, n_dn: int = 6, U: float = 4.0,
               steps: int = FLUX_STEPS, mode: str = "fixed", response_steps: int = FLUX_RESPONSE_STEPS, seed: int = 0,
               rand: Optional[Sequence[float]] = None, timing: Optional[SweepTiming] = None,
               autotune: bool = False, batch: int = 1) -> List[FluxPoint]:
    """E0(Phi), dE0/dPhi, d2E0/dPhi2 of Kagome12 (complex operator at every
    Phi, Phi = 0 included, so the second-order response sees the current).
    At twists where the operator is real a second ground state from another
    start vector tests the ground level for a two-fold degeneracy (the zero
    twist of the 6+6 sector is one); a degenerate level gets the derivatives
    of its lowest branch from ed_response_subspace.
    autotune: time the Lanczos kernel choices on the first twist's operator
    and apply the fastest to every twist (same shape, same tables).
    batch > 1 (fixed-step mode): up to `batch` (<= 16) twists share one
    persistent Lanczos launch for their ground states and one for their
    response solves (ed_lanczos_batch, ed_response_batch); the same start
    vectors, so the same results bit for bit.  batch = 0: the size
    tune_batch picks for this shape."""
    phis = flux_phis() if phis is None else phis
    t = timing if timing is not None else SweepTiming()
    if batch == 0 and mode == "fixed":  # the autotuner's batch size for this shape
        sample = []
        for phi in flux_phis(16):  # the sixteen-twist grid, whatever subset is swept
            terms = L.kagome12(rand, flux=float(phi), peierls=True)
            sample.append(Hubbard(H_TBq(12, n_up).extend(terms), H_TBq(12, n_dn).extend(terms), U))
        batch = tune_batch(sample)
        for op in sample:
            op.close()
    if batch > 1 and mode == "fixed":
        t0 = time.perf_counter()
        out = _flux_batched(list(phis), n_up, n_dn, U, steps, response_steps, seed, rand, min(batch, 16), t)
        t.total_s += time.perf_counter() - t0
        return out
    out: List[FluxPoint] = []
    tuned = None
    t0 = time.perf_counter()
    for k, phi in enumerate(phis):
        ti = time.perf_counter()
        terms = L.kagome12(rand, flux=float(phi), peierls=True)
        d1t, d2t = L.kagome12_flux_derivatives(float(phi), rand)
        H = Hubbard(H_TBq(12, n_up).extend(terms), H_TBq(12, n_dn).extend(terms), U)
        if autotune:
            if tuned is None:
                tuned = H.autotune(steps=30)["result"]
            else:
                H.set_tuning(tuned)
        dH = Hubbard(H_TBq(12, n_up).extend(d1t), H_TBq(12, n_dn).extend(d1t), 0.0)
        d2H = Hubbard(H_TBq(12, n_up).extend(d2t), H_TBq(12, n_dn).extend(d2t), 0.0)
        _sync()
        tb = time.perf_counter()
        e0, psi, n, bits = _ground(H, steps, mode, seed * 4096 + k)
        _sync()
        tl = time.perf_counter()
        states = [psi]
        if _real_twist(float(phi)):
            states = ground_multiplet(H, psi, e0, steps, mode, seed * 4096 + k)
        if len(states) > 1:
            import torch
            D1, M = ob.response_subspace(H, dH, d2H, torch.stack(states), e0, steps=response_steps)
            d1, d2 = ob.lowest_branch(D1, M)
        else:
            d1, d2 = ob.response(H, dH, d2H, psi, e0, steps=response_steps)
        _sync()
        te = time.perf_counter()
        for op in (H, dH, d2H):
            op.close()
        out.append(FluxPoint(float(phi), e0, d1, d2, n, bits))
        t.instances += 1
        t.lanczos_steps += n
        t.build_s += tb - ti
        t.lanczos_s += tl - tb
        t.observables_s += te - tl
        t.per_instance.append(te - ti)
    t.total_s += time.perf_counter() - t0
    return out


def ground_multiplet(H: Hubbard, psi, e0: float, steps: int, mode: str, seed: int, max_states: int = 4):
    """The ground level's states as far as Lanczos runs from further start
    vectors find new directions: each run whose Ritz value equals E0 (1e-10)
    and whose state keeps more than 1e-4 of its norm outside the span of the
    states found so far adds it; the first run that adds nothing ends the
    search.  A non-degenerate level costs one extra run."""
    states = [psi]
    for extra in range(1, max_states):
        e0b, psib, _, _ = _ground(H, steps, mode, seed + 2048 * extra)
        if abs(e0b - e0) > 1e-10 * abs(e0):
            break
        g = len(states)
        G = np.empty((g, g), dtype=np.complex128)
        for i in range(g):
            for j in range(g):
                G[i, j] = complex(*_zdot(states[i], states[j]))
        c = np.array([complex(*_zdot(states[i], psib)) for i in range(g)])
        nb = complex(*_zdot(psib, psib)).real
        outside = nb - float(np.real(np.vdot(c, np.linalg.solve(G, c))))
        if not outside > 1e-8 * nb:  # 1e-4 of the norm
            break
        states.append(psib)
    return states


def _zdot(x, y):
    """<x|y> of two CUDA tensors through the library (re, im)."""
    from ._capi import load
    out = np.zeros(2)
    n = x.numel()
    if x.is_complex():
        check_ = load().ed_vec_zdot(int(n), C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), 1,
                                    C.c_void_p(out.ctypes.data), None)
    else:
        check_ = load().ed_vec_dot(int(n), C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), 1,
                                   C.c_void_p(out.ctypes.data), None)
    if check_ != 0:
        from ._capi import EdError
        raise EdError(check_, "ed_vec_(z)dot")
    return out[0], out[1]


def _flux_batched(phis, n_up, n_dn, U, steps, response_steps, seed, rand, batch, t) -> List[FluxPoint]:
    import torch
    from ._capi import load
    lib = load()
    out: List[FluxPoint] = []
    for g0 in range(0, len(phis), batch):
        group = [(g0 + i, float(p)) for i, p in enumerate(phis[g0:g0 + batch])]
        ti = time.perf_counter()
        Hs, dHs, d2Hs = [], [], []
        for k, phi in group:
            terms = L.kagome12(rand, flux=phi, peierls=True)
            d1t, d2t = L.kagome12_flux_derivatives(phi, rand)
            Hs.append(Hubbard(H_TBq(12, n_up).extend(terms), H_TBq(12, n_dn).extend(terms), U))
            dHs.append(Hubbard(H_TBq(12, n_up).extend(d1t), H_TBq(12, n_dn).extend(d1t), 0.0))
            d2Hs.append(Hubbard(H_TBq(12, n_up).extend(d2t), H_TBq(12, n_dn).extend(d2t), 0.0))
        sizes = [2 * H.rows() for H in Hs]
        offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        starts = torch.empty(int(offs[-1]), dtype=torch.float64, device="cuda")
        for (k, _), o, n in zip(group, offs, sizes):
            lib.ed_random_vector_device(int(n), seed * 4096 + k, C.c_void_p(starts[int(o)].data_ptr()), None)
        evecs = torch.empty_like(starts)
        _sync()
        tb = time.perf_counter()
        results: list = []
        e0s, views, _, _ = lanczos_multi(Hs, steps, starts=starts, evec_out=evecs, results=results)
        _sync()
        tl = time.perf_counter()
        d1s, d2s, normal = [0.0] * len(group), [0.0] * len(group), []
        for i, (k, phi) in enumerate(group):
            if _real_twist(phi):
                states = ground_multiplet(Hs[i], views[i], float(e0s[i]), steps, "fixed", seed * 4096 + k)
                if len(states) > 1:
                    D1, M = ob.response_subspace(Hs[i], dHs[i], d2Hs[i], torch.stack(states), float(e0s[i]),
                                                 steps=response_steps)
                    d1s[i], d2s[i] = ob.lowest_branch(D1, M)
                    continue
            normal.append(i)
        if normal:
            psis = torch.cat([evecs[int(offs[i]):int(offs[i + 1])] for i in normal])
            f, sec = ob.response_batch([Hs[i] for i in normal], [dHs[i] for i in normal], [d2Hs[i] for i in normal],
                                       psis, [float(e0s[i]) for i in normal], steps=response_steps)
            for j, i in enumerate(normal):
                d1s[i], d2s[i] = float(f[j]), float(sec[j])
        _sync()
        te = time.perf_counter()
        for i, (k, phi) in enumerate(group):
            out.append(FluxPoint(phi, float(e0s[i]), d1s[i], d2s[i], steps, int(results[i].min_bits)))
        for op in Hs + dHs + d2Hs:
            op.close()
        t.instances += len(group)
        t.lanczos_steps += steps * len(group)
        t.build_s += tb - ti
        t.lanczos_s += tl - tb
        t.observables_s += te - tl
        t.per_instance.extend([(te - ti) / len(group)] * len(group))
    return out


def mbl_disorder(realisation: int, n_sites: int = 12, W: float = 6.0, seed: int = 0) -> Tuple[np.ndarray, np.ndarray]:
    """(eps_up, eps_dn) = W * uniform(-1, 1), 2 * n_sites numbers from
    Philox4x64-10 keyed by seed * 2^20 + realisation: the first n_sites for
    the up operator, the next for the down operator (the order of the two
    Line16 calls of Hubbard_EE_test.cu:68-69)."""
    x = random_vector(2 * n_sites, seed * (1 << 20) + realisation) * W
    return x[:n_sites].copy(), x[n_sites:].copy()


def mbl_chain_terms(eps: Sequence[float], t: float = -1.0):
    """Open chain with hopping t and on-site energies eps (Line16's bonds,
    Hubbard_EE_test.cu:119-139, for len(eps) sites)."""
    return L.chain(len(eps), t=t, periodic=False, eps=list(eps))


MBL_SECTORS = ((6, 6), (7, 5), (8, 4))


# Batch sizes chosen by tune_batch, per operator shape (n_sites, N_up, N_dn, complex).
_BATCH_CHOICE: dict = {}


def tune_batch(ops: Sequence[Hubbard], sizes=(1, 2, 4, 8, 16), steps: int = 60) -> int:
    """The number of Lanczos runs per persistent launch (ed_lanczos_batch)
    that gives the shortest time per run on these operators (one shape):
    each candidate runs len(ops) short fixed-step solves in groups of that
    size (a warm-up, then the better of two timed passes).  The choice is
    kept per shape for the rest of the process."""
    op0 = ops[0]
    key = (op0.N, op0.dimUP, op0.dimDN, op0.is_complex, len(op0._up_terms))
    if key in _BATCH_CHOICE:
        return _BATCH_CHOICE[key]
    best, pick = float("inf"), 1
    for bsz in sizes:
        if bsz > len(ops):
            break
        dt = float("inf")
        for rep in range(3):
            _sync()
            t0 = time.perf_counter()
            for g0 in range(0, len(ops), bsz):
                grp = list(ops[g0:g0 + bsz])
                if bsz == 1:
                    Lanczos().eigen(grp[0], max_steps=steps, mode="fixed", ritz="none", seed=g0)
                else:
                    lanczos_multi(grp, steps, ritz=False, seed=g0)
            _sync()
            if rep:
                dt = min(dt, time.perf_counter() - t0)
        if dt < best:
            best, pick = dt, bsz
    _BATCH_CHOICE[key] = pick
    return pick


def batch_choices() -> dict:
    """The batch sizes tune_batch has chosen so far, by shape."""
    return {f"N={k[0]} {k[1]}x{k[2]}{' complex' if k[3] else ''}": v for k, v in _BATCH_CHOICE.items()}


def _mbl_batched(reals, sectors, n_sites, W, U, steps, seed, a_sites, batch, t) -> List[MblPoint]:
    """mbl_sweep with the realisations of each sector in batches of `batch`
    Lanczos runs per persistent launch (ed_lanczos_batch); a sector the
    batched kernel does not take runs instance by instance.  Same start
    vectors, so the same results bit for bit."""
    import torch
    from ._capi import EdError, load
    lib = load()
    out: List[MblPoint] = []
    reals = list(reals)
    for s, (qu, qd) in enumerate(sectors):
        bsec = batch
        if batch <= 0:  # the autotuner's batch size for this sector, from eight fixed realisations
            sample = []
            for r in range(8):
                eu, edn = mbl_disorder(r, n_sites, W, seed)
                sample.append(Hubbard(H_TBq(n_sites, qu).extend(mbl_chain_terms(eu)),
                                      H_TBq(n_sites, qd).extend(mbl_chain_terms(edn)), U))
            bsec = tune_batch(sample, sizes=(1, 2, 4, 8))
            for op in sample:
                op.close()
        for g0 in range(0, len(reals), bsec):
            group = reals[g0:g0 + bsec]
            ti = time.perf_counter()
            ops = []
            for r in group:
                eu, edn = mbl_disorder(r, n_sites, W, seed)
                ops.append(Hubbard(H_TBq(n_sites, qu).extend(mbl_chain_terms(eu)),
                                   H_TBq(n_sites, qd).extend(mbl_chain_terms(edn)), U))
            _sync()
            tb = time.perf_counter()
            n = ops[0].rows()
            starts = torch.empty((len(ops), n), dtype=torch.float64, device="cuda")
            for b, r in enumerate(group):
                lib.ed_random_vector_device(n, seed * (1 << 20) + r * len(sectors) + s,
                                            C.c_void_p(starts[b].data_ptr()), None)
            evecs = torch.empty_like(starts)
            results: list = []
            try:
                e0s, _, _, _ = lanczos_batch(ops, steps, starts=starts, evec_out=evecs, results=results)
                bits = [int(r.min_bits) for r in results]
            except EdError:
                e0s, bits = [], []
                for b, op in enumerate(ops):
                    lz = Lanczos()
                    e, _ = lz.eigen(op, max_steps=steps, mode="fixed", ritz="stored",
                                    f=starts[b].cpu().numpy(), evec_out=evecs[b])
                    e0s.append(e)
                    bits.append(int(lz.result.min_bits))
            _sync()
            tl = time.perf_counter()
            # the group's entropies in one batched call (its blocks fill the GPU together)
            svns, srefs = ob.entanglement_entropy_batch(ops[0], evecs, a_sites)
            for b, r in enumerate(group):
                nu, nd, _ = ob.site_densities(ops[b], evecs[b])
                out.append(MblPoint(int(r), (qu, qd), float(e0s[b]), float(svns[b]), float(srefs[b]), nu, nd, steps,
                                    bits[b]))
            _sync()
            te = time.perf_counter()
            for op in ops:
                op.close()
            t.instances += len(group)
            t.lanczos_steps += steps * len(group)
            t.build_s += tb - ti
            t.lanczos_s += tl - tb
            t.observables_s += te - tl
            t.per_instance.extend([(te - ti) / len(group)] * len(group))
    order = {(r, sec): k for k, (r, sec) in enumerate((r, sec) for r in reals for sec in sectors)}
    return sorted(out, key=lambda p: order[(p.realisation, p.sector)])


def mbl_sweep(n_real: int = 64, sectors: Sequence[Tuple[int, int]] = MBL_SECTORS, n_sites: int = 12,
              W: float = 6.0, U: float = 1.0, steps: int = 300, mode: str = "fixed", seed: int = 0,
              a_sites: Optional[Sequence[int]] = None, realisations: Optional[Sequence[int]] = None,
              timing: Optional[SweepTiming] = None, batch: int = 1) -> List[MblPoint]:
    """Ground-state sweep over disorder realisations and sectors; batch > 1
    (fixed-step mode) runs up to 8 realisations of a sector per launch, batch
    = 0 the number tune_batch picks for each sector."""
    a_sites = list(range(n_sites // 2)) if a_sites is None else list(a_sites)
    reals = range(n_real) if realisations is None else realisations
    t = timing if timing is not None else SweepTiming()
    t0 = time.perf_counter()
    if (batch > 1 or batch == 0) and mode == "fixed":
        out = _mbl_batched(reals, sectors, n_sites, W, U, steps, seed, a_sites, min(batch, 8), t)
        t.total_s += time.perf_counter() - t0
        return out
    out: List[MblPoint] = []
    for r in reals:
        eu, edn = mbl_disorder(r, n_sites, W, seed)
        tu, td = mbl_chain_terms(eu), mbl_chain_terms(edn)
        for s, (qu, qd) in enumerate(sectors):
            ti = time.perf_counter()
            H = Hubbard(H_TBq(n_sites, qu).extend(tu), H_TBq(n_sites, qd).extend(td), U)
            _sync()
            tb = time.perf_counter()
            e0, psi, n, bits = _ground(H, steps, mode, seed * (1 << 20) + r * len(sectors) + s)
            _sync()
            tl = time.perf_counter()
            nu, nd, _ = ob.site_densities(H, psi)
            svn, sref = ob.entanglement_entropy(H, psi, a_sites)
            _sync()
            te = time.perf_counter()
            H.close()
            out.append(MblPoint(int(r), (qu, qd), e0, svn, sref, nu, nd, n, bits))
            t.instances += 1
            t.lanczos_steps += n
            t.build_s += tb - ti
            t.lanczos_s += tl - tb
            t.observables_s += te - tl
            t.per_instance.append(te - ti)
    t.total_s += time.perf_counter() - t0
    return out


def attach_oracle(points, oracle_e0) -> float:
    """Set err_vs_oracle = |E0 - oracle_e0[key]| on the points the table
    covers (key: round(Phi, 12) for twist points, (realisation, (N_up, N_dn))
    for disorder points); returns the largest such error (nan if none)."""
    worst = float("nan")
    for p in points:
        key = round(p.phi, 12) if isinstance(p, FluxPoint) else (p.realisation, tuple(p.sector))
        if key in oracle_e0:
            p.err_vs_oracle = abs(p.e0 - float(oracle_e0[key]))
            worst = p.err_vs_oracle if not worst >= p.err_vs_oracle else worst
    return worst


def flux_rows(points: Sequence[FluxPoint]):
    """Rows (Phi, E0, dE0/dPhi, d2E0/dPhi2, min_bits, |E0 - E0_oracle|) for
    datio.append_rows (nan where no oracle value was attached)."""
    return [(p.phi, p.e0, p.d1, p.d2, p.min_bits, p.err_vs_oracle) for p in points]


def mbl_rows(points: Sequence[MblPoint]):
    """Rows (realisation, N_up, N_dn, E0, S_vN, n_up[0..L-1], n_dn[0..L-1],
    min_bits, |E0 - E0_oracle|)."""
    return [(p.realisation, p.sector[0], p.sector[1], p.e0, p.s_vn) + tuple(p.n_up) + tuple(p.n_dn)
            + (p.min_bits, p.err_vs_oracle) for p in points]


FLUX_HEADER = "#       Phi       E0        dE0/dPhi        d2E0/dPhi2      min_bits        err_vs_oracle   "
MBL_HEADER = ("#       xid       Nup       Ndn       E0        S_A       n_up(i)...      n_dn(i)...      "
              "min_bits        err_vs_oracle   ")


# The plain per-instance GPU form the tuned sweep is compared with: the
# generic matvec kernel, host-driven per-step Lanczos launches, and one
# cusolverDnDgesvd per entanglement block on one stream.
PLAIN_ENV = {"ED_MATVEC": "generic", "ED_LZ_FUSED": "0", "ED_EE_METHOD": "gesvd", "ED_EE_STREAMS": "1"}
# The same plain Lanczos form with the tuned entanglement path (cluster
# bidiagonalisation), so that a comparison shows what batching, the
# persistent kernel and the row engine buy on their own.
PLAIN_SAME_EE_ENV = {"ED_MATVEC": "generic", "ED_LZ_FUSED": "0"}
FORM_ENV = {"tuned": {}, "plain": PLAIN_ENV, "plain_same_ee": PLAIN_SAME_EE_ENV}


def run_form(what: str, n: int, form: str, steps: Optional[int] = None, mode: str = "fixed", seed: int = 0,
             warmup: int = 1, batch: int = 0):
    """One sweep (what = "flux" | "mbl") in one form of FORM_ENV: the tuned
    form batches twists and disorder realisations (batch per launch; 0: the
    autotuner's size for each shape, tune_batch), the plain forms run one
    instance per launch sequence.  steps: Lanczos steps per instance (None: FLUX_STEPS
    for twists, 300 for disorder samples).  Returns (points, SweepTiming)."""
    if steps is None:
        steps = FLUX_STEPS if what == "flux" else 300
    import os
    env = FORM_ENV[form]
    keys = set(PLAIN_ENV) | set(env)
    saved = {k: os.environ.get(k) for k in keys}
    for k in keys:
        os.environ.pop(k, None)
    os.environ.update(env)
    try:
        tm = SweepTiming()
        if what == "flux":
            fb = batch if form == "tuned" else 1
            if warmup:
                flux_sweep(flux_phis(n)[:max(warmup, 2)], steps=steps, mode=mode, seed=seed, batch=fb)
            pts = flux_sweep(flux_phis(n), steps=steps, mode=mode, seed=seed, timing=tm, batch=fb)
        else:
            bt = batch if form == "tuned" else 1
            if warmup:
                mbl_sweep(realisations=range(max(warmup, bt)), steps=steps, mode=mode, seed=seed + 1, batch=bt)
            pts = mbl_sweep(n, steps=steps, mode=mode, seed=seed, timing=tm, batch=bt)
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    return pts, tm


def _run(a, n, form: str):
    return run_form(a.what, n, form, steps=a.steps, mode=a.mode, seed=a.seed, warmup=a.warmup, batch=a.batch)


def main(argv: Optional[Sequence[str]] = None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--what", choices=["flux", "mbl"], default="mbl")
    ap.add_argument("--n", type=int, default=None, help="flux points (16) or realisations (64)")
    ap.add_argument("--steps", type=int, default=None, help="Lanczos steps (default: 500 twists, 300 disorder)")
    ap.add_argument("--mode", choices=["fixed", "reference"], default="fixed")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--warmup", type=int, default=1, help="instances run (untimed) before the sweep")
    ap.add_argument("--out", default=None, help="append the result rows to this .dat file")
    ap.add_argument("--batch", type=int, default=0,
                    help="runs per Lanczos launch in the tuned form (0: the autotuner's choice per shape, "
                         "1: one launch per run)")
    ap.add_argument("--form", choices=["tuned", "plain", "plain_same_ee", "compare"], default="tuned",
                    help="plain: the per-instance form of PLAIN_ENV; plain_same_ee: the same with the tuned "
                         "entanglement path; compare: tuned and plain, with the largest differences of their "
                         "outputs")
    a = ap.parse_args(argv)
    import torch
    if not torch.cuda.is_available():
        raise SystemExit("sweeps need a CUDA device")
    if a.what == "flux":
        n = 16 if a.n is None else a.n
        cfg = {"workload": f"Kagome12 6+6 U=4, {n} twists in [0, 2pi/{L.KAGOME12_LX:g}], complex FP64",
               "lanczos_steps": a.steps, "response_steps": 200, "mode": a.mode}
    else:
        n = 64 if a.n is None else a.n
        cfg = {"workload": f"open chain L=12 t=1 U=1 W=6, {n} realisations x sectors (6,6),(7,5),(8,4)",
               "lanczos_steps": a.steps, "mode": a.mode, "entanglement_sites": "0..5"}
    forms = ["tuned", "plain"] if a.form == "compare" else [a.form]
    runs = {f: _run(a, n, f) for f in forms}
    pts, tm = runs[forms[0]]
    rows, header = (flux_rows(pts), FLUX_HEADER) if a.what == "flux" else (mbl_rows(pts), MBL_HEADER)
    if a.out:
        from .datio import append_rows
        append_rows(a.out, header, rows)
    line = {"sweep": a.what, "form": forms[0], "config": cfg, **tm.summary(),
            "ms_per_instance_median": round(1e3 * float(np.median(tm.per_instance)), 3)}
    if a.form == "compare":
        p_pts, p_tm = runs["plain"]
        diff = np.abs(np.array(rows, dtype=float)[:, :-2] -
                      np.array(flux_rows(p_pts) if a.what == "flux" else mbl_rows(p_pts), dtype=float)[:, :-2])
        line["plain"] = p_tm.summary()
        line["speedup_vs_plain"] = round(p_tm.total_s / tm.total_s, 3)
        line["max_abs_diff_vs_plain"] = {"E0": float(np.max(diff[:, 1 if a.what == "flux" else 3])),
                                         "all_columns": float(np.max(diff))}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
