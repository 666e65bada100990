"""tf_solve_bsr_static: the linear solve for callers that cannot allocate
device memory (their host owns every device allocation, or they run under a
fixed memory budget).  It must agree with the solve behind tf_solve on the
same system, on two calls in a row (the static work space is reused), leave
the device's free memory unchanged on the second call, reject systems larger
than its static limit and refuse a stream that is being captured.

The test allocates device memory itself (through torch) to hold the
caller-owned matrix and vectors; only the entry point under test must not.
It lives in its own file so pytest collects it after every other test.
"""
import ctypes as C

import numpy as np
import pytest

from tissuefolding_paperversion_gb300 import api, mesh

pytestmark = pytest.mark.gpu
TOL = 1e-8  # the position tolerance of the parity tests


def _bsr_of_transpose(ia, ja, a, n_nodes):
    """Block-sparse rows of A = K^T from the reference-layout CSR of K."""
    rows = np.repeat(np.arange(len(ia) - 1), np.diff(ia))
    r, c = ja, rows                      # A[r][c] = K[c][r]
    br, bc = r // 3, c // 3
    key = br.astype(np.int64) * n_nodes + bc
    order = np.unique(key)
    rowptr = np.zeros(n_nodes + 1, dtype=np.int32)
    np.add.at(rowptr, (order // n_nodes) + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    colidx = (order % n_nodes).astype(np.int32)
    blk = np.searchsorted(order, key)
    val = np.zeros((len(order), 9))
    val[blk, 3 * (r % 3) + (c % 3)] = a
    return rowptr, colidx, val.reshape(-1)


@pytest.mark.parametrize("eta", [0.0, 100.0])
def test_static_solve_matches_tf_solve_twice(eta):
    torch = pytest.importorskip("torch")
    t = mesh.config_small(seed=7)
    t.eta[:] = eta
    uk, un = mesh.perturbed_state(t, seed=8, amp=0.1)
    # a firm viscosity surface keeps the system well conditioned, so two
    # solves stopped at the same small residual agree to the tolerance
    with api.Solver(t, krylov_rtol=1e-13) as s:
        s.set_state(uk, un, t.dt)
        s.set_viscosity_surfaces(np.full(t.n_nodes, 100.0))
        s.assemble()
        ia, ja, a = s.export_csr(0.0)
        g = s.residual()
        ref = s.solve()
        du_ref = s.delta_u()
    assert ref["relres"] <= 1e-13
    rowptr, colidx, val = _bsr_of_transpose(ia, ja, a, t.n_nodes)
    dev = torch.device("cuda:0")
    d_rowptr = torch.from_numpy(rowptr).to(dev)
    d_colidx = torch.from_numpy(colidx).to(dev)
    d_val = torch.from_numpy(val).to(dev)
    d_b = torch.from_numpy(g).to(dev)
    L = api.load()
    d_xs = [torch.full((3 * t.n_nodes,), float("nan"), dtype=torch.float64, device=dev) for _ in range(2)]
    torch.cuda.synchronize()
    for call, d_x in enumerate(d_xs):
        free_before = torch.cuda.mem_get_info(dev)[0]
        it, rr = C.c_int32(0), C.c_double(0.0)
        st = L.tf_solve_bsr_static(t.n_nodes, C.c_void_p(d_rowptr.data_ptr()), C.c_void_p(d_colidx.data_ptr()),
                                   C.c_void_p(d_val.data_ptr()), C.c_void_p(d_b.data_ptr()),
                                   C.c_void_p(d_x.data_ptr()), 1e-13, 20000, None, C.byref(it), C.byref(rr))
        assert st == api.TF_OK, L.tf_last_error().decode()
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info(dev)[0]
        if call == 1:
            # the first call may still page in the library's static array and the
            # kernels' local memory; the second must not take any device memory
            assert free_after == free_before, (free_before, free_after)
        x = d_x.cpu().numpy()
        assert rr.value <= 1e-13 and it.value > 0
        assert np.abs(x - du_ref).max() <= TOL * np.abs(du_ref).max(), call


def test_static_solve_refuses_a_capturing_stream():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    n = 4
    rowptr = torch.arange(n + 1, dtype=torch.int32, device=dev)
    colidx = torch.arange(n, dtype=torch.int32, device=dev)
    val = torch.eye(3, dtype=torch.float64, device=dev).reshape(-1).repeat(n)
    b = torch.ones(3 * n, dtype=torch.float64, device=dev)
    x = torch.zeros(3 * n, dtype=torch.float64, device=dev)
    y = torch.zeros(1, device=dev)
    L = api.load()
    it, rr = C.c_int32(0), C.c_double(0.0)
    side = torch.cuda.Stream(device=dev)
    graph = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(graph, stream=side):
        y.add_(1.0)
        st = L.tf_solve_bsr_static(n, C.c_void_p(rowptr.data_ptr()), C.c_void_p(colidx.data_ptr()),
                                   C.c_void_p(val.data_ptr()), C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()),
                                   1e-10, 10, C.c_void_p(side.cuda_stream), C.byref(it), C.byref(rr))
    assert st == api.TF_BAD_INPUT
    assert "captured" in L.tf_last_error().decode()
    # the capture was left intact: the graph replays
    graph.replay()
    torch.cuda.synchronize()
    assert float(y.item()) == 1.0
    # and the same call outside a capture solves the identity system
    st = L.tf_solve_bsr_static(n, C.c_void_p(rowptr.data_ptr()), C.c_void_p(colidx.data_ptr()),
                               C.c_void_p(val.data_ptr()), C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()),
                               1e-10, 10, None, C.byref(it), C.byref(rr))
    assert st == api.TF_OK, L.tf_last_error().decode()
    assert np.allclose(x.cpu().numpy(), 1.0)


def test_static_solve_rejects_oversized_system():
    L = api.load()
    it, rr = C.c_int32(0), C.c_double(0.0)
    fake = C.c_void_p(16)   # never dereferenced: the size check comes first
    st = L.tf_solve_bsr_static(16385, fake, fake, fake, fake, fake, 1e-10, 10, None, C.byref(it), C.byref(rr))
    assert st == api.TF_BAD_INPUT
    assert "static limit" in L.tf_last_error().decode()
