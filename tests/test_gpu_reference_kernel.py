"""The reference's own GPU matvec (Hubbard_mv_, HubMatrix_GPU.cuh:114-161,
compiled unmodified into oracle/_ref/ref_mv.cubin) as a second checker and a
same-GPU baseline.

Parity: on every real operator of the matvec suite the library's y = H x and
the reference kernel's differ by less than 1e-13 normwise relative (the
reference sums its FP64 products in slot order with one rounding each; the
library sums exactly and rounds once).  Timing: both kernels on the same
device vectors, CUDA events on the launching stream, back-to-back calls
after warm-up (the vectors of these sizes stay in L2 for both).

Skipped when the cubin was not built (it is built from the reference
checkout by `make -C oracle ref`).
"""
import numpy as np
import pytest

from conftest import rel_err
from test_gpu_matvec import make_op, real_cases

pytestmark = pytest.mark.gpu
TOL = 1e-13


@pytest.fixture(scope="module")
def refk():
    from oracle import refkernel
    if not refkernel.available():
        pytest.skip("oracle/_ref/ref_mv.cubin not built (needs the reference checkout)")
    return refkernel


def _pair(ed, refk, case):
    name, N, qu, qd, ut, dt, U, dil = case
    try:
        ref = refk.RefHubbard(ed.H_TBq(N, qu).extend(ut), ed.H_TBq(N, qd).extend(dt), U, dilution=dil)
    except ValueError as e:  # shapes the reference kernel does not handle (fewer down states than up slots)
        pytest.skip(f"{name}: {e}")
    return make_op(ed, N, qu, qd, ut, dt, U, dil), ref


@pytest.mark.parametrize("case", real_cases(), ids=lambda c: c[0])
def test_matvec_vs_reference_kernel(ed, refk, case):
    import torch
    op, ref = _pair(ed, refk, case)
    rng = np.random.default_rng(17)
    x = torch.from_numpy(rng.uniform(-1.0, 1.0, op.rows())).cuda()
    y, yr = torch.empty_like(x), torch.empty_like(x)
    op.Hubbard_mv(x, y)
    ref(x, yr)
    torch.cuda.synchronize()
    assert ref.launches == 1
    assert rel_err(y.cpu().numpy(), yr.cpu().numpy()) < TOL, case[0]
    ref.close()
    op.close()


def _time_us(fn, reps=50, warm=5):
    import torch
    for _ in range(warm):
        fn()
    s = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(s)
    for _ in range(reps):
        fn()
    b.record(s)
    torch.cuda.synchronize()
    return a.elapsed_time(b) * 1e3 / reps


def test_reference_kernel_timing(ed, refk):
    """Prints µs per matvec for the reference kernel and the library's
    device-vector matvec (Hubbard_mv) on C1, C2 and the C4 sectors."""
    import torch
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import sweeps
    eu, edn = sweeps.mbl_disorder(0)
    cases = [("C1 chain8 pbc (4,4) U=4", 8, 4, 4, L.chain(8), L.chain(8), 4.0, None),
             ("C2 kagome12 (6,6) U=8", 12, 6, 6, L.kagome12(), L.kagome12(), 8.0, None)]
    for q in sweeps.MBL_SECTORS:
        cases.append((f"C4 chain12 open W=6 {q} U=1", 12, q[0], q[1], sweeps.mbl_chain_terms(eu),
                      sweeps.mbl_chain_terms(edn), 1.0, None))
    rows = []
    for case in cases:
        op, ref = _pair(ed, refk, case)
        x = torch.from_numpy(np.random.default_rng(3).uniform(-1.0, 1.0, op.rows())).cuda()
        y, yr = torch.empty_like(x), torch.empty_like(x)
        t_ref = _time_us(lambda: ref(x, yr))
        t_lib = _time_us(lambda: op.Hubbard_mv(x, y))
        torch.cuda.synchronize()
        err = rel_err(y.cpu().numpy(), yr.cpu().numpy())
        assert err < TOL, case[0]
        gbs = lambda us: 16.0 * op.rows() / (us * 1e-6) / 1e9  # noqa: E731
        rows.append((case[0], op.rows(), t_ref, t_lib, t_ref / t_lib, gbs(t_ref), gbs(t_lib), err))
        ref.close()
        op.close()
    print("\nconfig | D | reference Hubbard_mv_ us | library Hubbard_mv us | speed-up | ref GB/s | lib GB/s | rel diff")
    for r in rows:
        print(f"{r[0]} | {r[1]} | {r[2]:.1f} | {r[3]:.1f} | {r[4]:.2f} | {r[5]:.0f} | {r[6]:.0f} | {r[7]:.1e}")
