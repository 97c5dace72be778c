"""ed_op_perform_noalloc: the operator apply for callers that cannot let the
library allocate GPU memory — code whose device memory is owned by another
allocator (a framework's caching pool that has already reserved the GPU), and
loops that cannot take the implicit synchronisation of cudaMalloc/cudaFree.
Its scratch is a fixed static device array.

Checked through the C ABI: on freshly created operators (so that nothing
allocated by ed_op_perform can stand in for the scratch) two calls in a row
match the FP64 oracle and then ed_op_perform (tolerance 1e-13 normwise, the
matvec tolerance of the other tests), the second call is not affected by
what the first left in the shared scratch, the device's free memory is the
same before and after a call, and sizes beyond the array are refused.  It
sits in its own file, collected last, and passes both alone and after the
other tests."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _case(ed, case):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    if case == "kagome12_66_real":
        t, q, U = L.kagome12(), 6, 8.0
    else:
        t, q, U = L.kagome12(flux=0.3), 5, 4.0
    return t, q, U, ed.Hubbard(ed.H_TBq(12, q).extend(t), ed.H_TBq(12, q).extend(t), U)


def _oracle_apply(orc, t, q, U, x):
    """y = H x on the CPU: the restated Hubbard_mv_ for real terms, the
    Kronecker-sum construction for Peierls phases."""
    if np.iscomplexobj(x):
        return orc.hamiltonian(12, q, q, t, t, U) @ x
    tab = orc.Tables(12, q, t)
    return orc.matvec(tab, tab, U, x)


@pytest.mark.parametrize("case", ["kagome12_66_real", "kagome12_55_flux"])
def test_noalloc_apply_matches_oracle_and_perform(ed, edlib, orc, case):
    import torch
    t, q, U, op = _case(ed, case)
    n = op.rows() * (2 if op.is_complex else 1)
    g = torch.Generator(device="cuda").manual_seed(5)
    for call in range(2):
        # the second input spans a very different magnitude, so a stale
        # exponent or flag from the first call would show
        scale = 1.0 if call == 0 else 2.0 ** -300
        x = torch.randn(n, dtype=torch.float64, device="cuda", generator=g) * scale
        y = torch.empty_like(x)
        y_ref = torch.empty_like(x)
        # the no-allocation entry first: the operator has not run any other apply yet
        assert edlib.ed_op_perform_noalloc(op.handle, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), None) == 0
        torch.cuda.synchronize()
        xh = x.cpu().numpy()
        yh = y.cpu().numpy()
        if op.is_complex:
            xh, yh = xh.view(np.complex128), yh.view(np.complex128)
        assert rel(yh, _oracle_apply(orc, t, q, U, xh)) < 1e-13
        assert edlib.ed_op_perform(op.handle, C.c_void_p(x.data_ptr()), C.c_void_p(y_ref.data_ptr()), 1, None) == 0
        torch.cuda.synchronize()
        assert rel(y.cpu().numpy(), y_ref.cpu().numpy()) < 1e-13
    op.close()


def test_noalloc_first_call_leaves_free_memory_unchanged(ed, edlib):
    """After one warm-up call on another operator of the same kind (which
    loads the kernels and resolves the scratch address), the first call on a
    fresh operator changes the device's free memory by nothing."""
    import torch
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    t = L.kagome12()
    warm = ed.Hubbard(ed.H_TBq(12, 6).extend(t), ed.H_TBq(12, 6).extend(t), 4.0)
    x = torch.randn(warm.rows(), dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    assert edlib.ed_op_perform_noalloc(warm.handle, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), None) == 0
    op = ed.Hubbard(ed.H_TBq(12, 6).extend(t), ed.H_TBq(12, 6).extend(t), 8.0)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    assert edlib.ed_op_perform_noalloc(op.handle, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), None) == 0
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0, (free0, free1)
    assert torch.isfinite(y).all()
    warm.close()
    op.close()


def test_noalloc_rejects_oversized_operator(ed, edlib):
    import torch
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    op = ed.Hubbard(ed.H_TBq(14, 7).extend(L.chain(14)), ed.H_TBq(14, 7).extend(L.chain(14)), 1.0)
    assert op.rows() > (1 << 21)
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    assert edlib.ed_op_perform_noalloc(op.handle, C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()), None) == 5
    op.close()
