"""ed_op_perform_noalloc: the operator apply for callers that cannot let the
library allocate GPU memory (device memory owned by another allocator, or
loops that cannot take the implicit synchronisation of cudaMalloc/cudaFree).
Its scratch is a fixed static device array; this test checks, through the C
ABI, that two calls in a row give the same result as ed_op_perform (tolerance
1e-13 normwise, the matvec tolerance of the other tests), that the second
call is not affected by what the first left in the shared scratch, and that
sizes beyond the array are refused.  It sits in its own file, collected last,
and passes both alone and after the other tests."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("case", ["kagome12_66_real", "kagome12_55_flux"])
def test_noalloc_apply_matches_perform(ed, edlib, case):
    import torch
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    if case == "kagome12_66_real":
        t, q, U = L.kagome12(), 6, 8.0
    else:
        t, q, U = L.kagome12(flux=0.3), 5, 4.0
    op = ed.Hubbard(ed.H_TBq(12, q).extend(t), ed.H_TBq(12, q).extend(t), U)
    n = op.rows() * (2 if op.is_complex else 1)
    g = torch.Generator(device="cuda").manual_seed(5)
    for call in range(2):
        # the second input spans a very different magnitude, so a stale
        # exponent or flag from the first call would show
        scale = 1.0 if call == 0 else 2.0 ** -300
        x = torch.randn(n, dtype=torch.float64, device="cuda", generator=g) * scale
        y_ref = torch.empty_like(x)
        y = torch.empty_like(x)
        assert edlib.ed_op_perform(op.handle, C.c_void_p(x.data_ptr()), C.c_void_p(y_ref.data_ptr()), 1, None) == 0
        assert edlib.ed_op_perform_noalloc(op.handle, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), None) == 0
        torch.cuda.synchronize()
        assert rel(y.cpu().numpy(), y_ref.cpu().numpy()) < 1e-13


def test_noalloc_rejects_oversized_operator(ed, edlib):
    import torch
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    op = ed.Hubbard(ed.H_TBq(14, 7).extend(L.chain(14)), ed.H_TBq(14, 7).extend(L.chain(14)), 1.0)
    assert op.rows() > (1 << 21)
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    assert edlib.ed_op_perform_noalloc(op.handle, C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()), None) == 5
