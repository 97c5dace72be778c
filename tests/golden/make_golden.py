"""Generate the golden fixtures in this directory.

Run from the repository root in a checkout where the reference sources are
available (they are read by oracle/Makefile's `ref` target, which compiles
the reference's own MBL_test/include/fermi_operator.h into
oracle/_ref/ref_tables):

    make -C oracle ref && python tests/golden/make_golden.py
    python tests/golden/make_golden.py --flux     (flux fixtures only; no
                                                   reference build needed)
    python tests/golden/make_golden.py --sweep    (disorder-sweep instances)

Outputs
  tables_small.npz   reference H_TBq state/Ax/Aj arrays for small cases
  tables_digest.json sha256 digests of the reference tables for large cases
  energies.json      ground-state energies (dense or scipy eigsh on the
                     reference tables) and entanglement entropies
  flux_kagome12_q66_U4.json
                     the twisted Kagome12 6+6, U=4 sector at three of the
                     sixteen twists Phi_k = (2 pi / 4) k / 15: E0 and E1
                     (scipy eigsh on the oracle's Kronecker-sum Hamiltonian
                     with the Peierls phases), dE0/dPhi = <psi|H'|psi> and
                     d2E0/dPhi2 = <psi|H''|psi> - 2 <b|(H - E0)^+|b>,
                     b = Q H' psi, from a projected conjugate-gradient solve
  sweep_chain12_W6.json
                     E0 of the first disorder realisations of the L=12 chain
                     sweep in its three sectors (scipy eigsh)
"""
from __future__ import annotations

import hashlib
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402
from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L  # noqa: E402

OUT = Path(__file__).resolve().parent


def digest(state, ax, aj) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(state, dtype=np.int64).tobytes())
    h.update(np.ascontiguousarray(ax, dtype=np.float64).tobytes())
    h.update(np.ascontiguousarray(aj, dtype=np.int64).tobytes())
    return h.hexdigest()


def disorder(seed: int, n: int, W: float) -> list:
    """eps_i = W * uniform(-1,1) from Philox4x64-10(key=seed) — the same
    stream ed_random_vector produces."""
    bg = np.random.Philox(key=np.array([seed, 0], dtype=np.uint64))
    r = bg.random_raw(n)
    u = ((r >> np.uint64(12)) | np.uint64(0x3FF0000000000000)).view(np.float64) * 2.0 - 3.0
    return [float(W * v) for v in u]


# name -> (N, Q, terms)
def cases_small():
    eps = disorder(11, 8, 2.0)
    return {
        "chain8_q4": (8, 4, L.chain(8)),
        "chain8_q3": (8, 3, L.chain(8)),
        "chain8_q4_open_eps": (8, 4, L.chain(8, periodic=False, eps=eps)),
        "chain8_q4_current": (8, 4, [("J", i, (i + 1) % 8, 1.0, 0.0) for i in range(8)]),
        "kagome12_q6": (12, 6, L.kagome12()),
        "kagome12_q5_kx": (12, 5, L.kagome12_kinetic_x()),
        "kagome12_q6_jx": (12, 6, L.kagome12_current_x()),
        "lieb12_q6": (12, 6, L.lieb12()),
        "square3x4_q3": (12, 3, L.squared_3by4()),
    }


def cases_large():
    out = {}
    for q in (6, 7, 8, 4, 5):
        out[f"chain12_open_q{q}_W6"] = (12, q, L.chain(12, periodic=False, eps=disorder(100, 12, 6.0)))
    out["lieb18_q9"] = (18, 9, L.lieb18())
    out["kagome12_q6_ky"] = (12, 6, L.kagome12_kinetic_y())
    out["kagome12_q6_jy"] = (12, 6, L.kagome12_current_y())
    return out


def main() -> None:
    if not O.REF_TABLES.exists():
        raise SystemExit("oracle/_ref/ref_tables missing: run `make -C oracle ref` first")
    small = {}
    meta = {}
    for name, (N, Q, terms) in cases_small().items():
        state, address, ax, aj = O.ref_tables(N, Q, terms)
        small[f"{name}__state"] = state.astype(np.int64)
        small[f"{name}__ax"] = ax
        small[f"{name}__aj"] = aj.astype(np.int32)
        meta[name] = {"N": N, "Q": Q, "terms": terms}
    np.savez_compressed(OUT / "tables_small.npz", **small)

    digests = {}
    for name, (N, Q, terms) in cases_large().items():
        t0 = time.time()
        state, address, ax, aj = O.ref_tables(N, Q, terms)
        digests[name] = {"N": N, "Q": Q, "terms": terms, "sha256": digest(state, ax, aj),
                         "count": int(state.size), "nnz": int((ax != 0).sum())}
        print(name, f"{time.time() - t0:.1f}s", flush=True)
    (OUT / "tables_digest.json").write_text(json.dumps({"small": meta, "large": digests}, indent=1))

    import scipy.sparse.linalg as sla
    en = {}
    # L=8 periodic chain, 4+4: dense spectrum
    for U in (4.0, 0.0):
        H = O.hamiltonian(8, 4, 4, L.chain(8), L.chain(8), U).toarray()
        w, v = np.linalg.eigh(H)
        en[f"chain8_pbc_q44_U{U:g}"] = {"E0": float(w[0]), "E1": float(w[1])}
        if U == 4.0:
            s_vn, s_ref = O.entanglement_entropy(v[:, 0], 8, 4, 4, [0, 1, 2, 3])
            en["chain8_pbc_q44_U4"].update({"EE_vN_A0123": s_vn, "EE_ref_A0123": s_ref})
    # atomic limit t=0 with site energies: E0 = min over configurations
    eps = disorder(11, 8, 2.0)
    H = O.hamiltonian(8, 3, 2, [("N", i, 0, eps[i], 0.0) for i in range(8)],
                      [("N", i, 0, eps[i], 0.0) for i in range(8)], 3.0)
    en["atomic8_q32_U3"] = {"E0": float(H.diagonal().min()), "eps": eps}
    # Kagome12 6+6 (reference lattice incl. the -2 r^2 on-site term), U=8 and U=4
    for U in (8.0, 4.0):
        t0 = time.time()
        H = O.hamiltonian(12, 6, 6, L.kagome12(), L.kagome12(), U)
        w = sla.eigsh(H, k=2, which="SA", tol=1e-13, maxiter=20000)[0]
        en[f"kagome12_q66_U{U:g}"] = {"E0": float(np.sort(w)[0]), "E1": float(np.sort(w)[1])}
        print("kagome", U, f"{time.time() - t0:.1f}s", flush=True)
    # Lieb12 6+6 U=4
    H = O.hamiltonian(12, 6, 6, L.lieb12(), L.lieb12(), 4.0)
    w = sla.eigsh(H, k=1, which="SA", tol=1e-13, maxiter=20000)[0]
    en["lieb12_q66_U4"] = {"E0": float(w[0])}
    # MBL chain L=12 open, W=6, U=1, one realisation, three sectors
    eps12 = disorder(100, 12, 6.0)
    for qu, qd in ((6, 6), (7, 5), (8, 4)):
        terms = L.chain(12, periodic=False, eps=eps12)
        H = O.hamiltonian(12, qu, qd, terms, terms, 1.0)
        w, v = sla.eigsh(H, k=1, which="SA", tol=1e-13, maxiter=20000)
        s_vn, s_ref = O.entanglement_entropy(v[:, 0], 12, qu, qd, list(range(6)))
        en[f"chain12_open_W6_seed100_q{qu}{qd}_U1"] = {"E0": float(w[0]), "EE_vN_A0to5": s_vn,
                                                       "EE_ref_A0to5": s_ref, "eps": eps12}
    (OUT / "energies.json").write_text(json.dumps(en, indent=1))
    print(json.dumps(en, indent=1))


def _projected_solve(H, e0, S, b):
    """phi with (Q (H - E0) Q + P) phi = b, P the projector on the columns of
    S (orthonormal), Q = 1 - P; b orthogonal to S.  Conjugate gradients."""
    import scipy.sparse.linalg as sla
    n = H.shape[0]

    def apply(x):
        x = np.asarray(x).reshape(-1)
        c = S.conj().T @ x
        xq = x - S @ c
        y = H @ xq - e0 * xq
        y = y - S @ (S.conj().T @ y)
        return y + S @ c

    A = sla.LinearOperator((n, n), matvec=apply, dtype=np.complex128)
    its = [0]

    def cb(_):
        its[0] += 1

    sol, info = sla.cg(A, b, rtol=1e-14, atol=0.0, maxiter=20000, callback=cb)
    if info != 0:
        raise RuntimeError(f"CG did not converge (info {info})")
    return sol, its[0], float(np.linalg.norm(apply(sol) - b) / np.linalg.norm(b))


def flux_fixtures(ks=(0, 7, 15), n_phi: int = 16) -> dict:
    """E0, dE0/dPhi, d2E0/dPhi2 of Kagome12 6+6, U=4 with the twist phase
    Phi * dx_b on every bond (KagomeCurrent12's x projections,
    drude_v2_cal_Kagome_randomHop.cu:849-851), on the CPU.

    Where the ground level is degenerate (at Phi = 0 it is two-fold), the
    derivatives are those of the lowest branch E0(Phi) by degenerate
    perturbation theory on the ground subspace S: the first-order matrix
    D1 = S^H H' S and, when D1 vanishes, the second-order matrix
    M = S^H H'' S - 2 B^H (Q (H - E0) Q)^+ B with B = Q H' S; d2E0/dPhi2 is
    the lowest eigenvalue of M.  Checked against E0(+-h), h = 1e-3."""
    import math
    import scipy.sparse.linalg as sla
    out = {"lattice": "Kagome12 (KagomeLattice12 incl. -2 r^2 on-site), r_i = 1", "n_up": 6, "n_dn": 6, "U": 4.0,
           "phi_k": "(2 pi / KAGOME12_LX) * k / 15, KAGOME12_LX = 4", "points": []}

    def ham(phi):
        terms = L.kagome12(flux=phi, peierls=True)
        return O.hamiltonian(12, 6, 6, terms, terms, 4.0)

    def lowest(H, k, seed):
        v0 = (np.random.default_rng(seed).standard_normal(H.shape[0])
              + 1j * np.random.default_rng(seed + 1).standard_normal(H.shape[0]))
        w, v = sla.eigsh(H, k=k, which="SA", tol=1e-14, maxiter=50000, v0=v0)
        o = np.argsort(w)
        return w[o], v[:, o]

    for k in ks:
        t0 = time.time()
        phi = (2.0 * math.pi / L.KAGOME12_LX) * k / (n_phi - 1)
        d1t, d2t = L.kagome12_flux_derivatives(phi)
        H = ham(phi)
        H1 = O.hamiltonian(12, 6, 6, d1t, d1t, 0.0)
        H2 = O.hamiltonian(12, 6, 6, d2t, d2t, 0.0)
        w, v = lowest(H, 4, k)
        e0 = float(w[0])
        g = int(np.sum(w - e0 < 1e-9 * abs(e0)))
        S, _ = np.linalg.qr(v[:, :g])
        HS = H1 @ S
        D1 = S.conj().T @ HS
        B = HS - S @ D1
        sols, its, res = [], [], []
        for i in range(g):
            x, it, r = _projected_solve(H, e0, S, B[:, i])
            sols.append(x)
            its.append(it)
            res.append(r)
        X = np.stack(sols, axis=1)
        M = S.conj().T @ (H2 @ S) - 2.0 * (B.conj().T @ X)
        M = 0.5 * (M + M.conj().T)
        d1_branches = np.linalg.eigvalsh(0.5 * (D1 + D1.conj().T))
        d2_branches = np.linalg.eigvalsh(M)
        rec = {"k": int(k), "phi": phi, "E0": e0, "E1": float(w[g]), "degeneracy": g,
               "dE0_dphi": float(d1_branches[0]), "d2E0_dphi2": float(d2_branches[0]),
               "dE0_dphi_branches": [float(x) for x in d1_branches],
               "d2E0_dphi2_branches": [float(x) for x in d2_branches],
               "eigsh_residual": float(np.linalg.norm(H @ v[:, 0] - e0 * v[:, 0])),
               "cg_iterations": its, "cg_rel_residual": max(res)}
        if g > 1:
            h = 1e-3
            ep = float(lowest(ham(phi + h), 2, 100 + k)[0][0])
            em = float(lowest(ham(phi - h), 2, 200 + k)[0][0])
            rec["d2E0_dphi2_fd_h1e-3"] = (ep + em - 2.0 * e0) / (h * h)
            rec["dE0_dphi_fd_h1e-3"] = (ep - em) / (2.0 * h)
        out["points"].append(rec)
        print(json.dumps(rec), f"{time.time() - t0:.1f}s", flush=True)
    return out


def sweep_fixtures(realisations=(0, 1), sectors=((6, 6), (7, 5), (8, 4)), W: float = 6.0, seed: int = 0) -> dict:
    """E0 of disorder-sweep instances (open L=12 chain, t=1, U=1, on-site
    W * uniform(-1,1) from Philox keyed by seed * 2^20 + realisation, the
    first 12 numbers for the up operator and the next 12 for the down one)
    by scipy eigsh on the oracle's Kronecker-sum Hamiltonian."""
    import scipy.sparse.linalg as sla
    out = {"workload": "open chain L=12, t=1, U=1, W=6", "points": []}
    for r in realisations:
        x = O.philox_uniform(seed * (1 << 20) + r, 24, W)
        tu = L.chain(12, periodic=False, eps=list(x[:12]))
        td = L.chain(12, periodic=False, eps=list(x[12:]))
        for qu, qd in sectors:
            t0 = time.time()
            H = O.hamiltonian(12, qu, qd, tu, td, 1.0)
            v0 = np.random.default_rng(r).standard_normal(H.shape[0])
            w = np.sort(sla.eigsh(H, k=2, which="SA", tol=1e-14, maxiter=50000, v0=v0)[0])
            out["points"].append({"realisation": int(r), "sector": [qu, qd], "E0": float(w[0]), "E1": float(w[1])})
            print(f"mbl r={r} ({qu},{qd}) E0={w[0]!r} gap={w[1] - w[0]:.3e} {time.time() - t0:.1f}s", flush=True)
    return out


if __name__ == "__main__":
    if "--sweep" in sys.argv[1:]:
        (OUT / "sweep_chain12_W6.json").write_text(json.dumps(sweep_fixtures(), indent=1))
    elif "--flux" in sys.argv[1:]:
        (OUT / "flux_kagome12_q66_U4.json").write_text(json.dumps(flux_fixtures(), indent=1))
    else:
        main()
