"""Partitioned partial-pivoting solve (WM-pGE, one CTA per system) against
the oracle: every partition-count variant, sizes around the partition
boundaries, the breakdown fallback (singular interior blocks) and LAPACK's
info for singular matrices.

Tolerances: normwise backward error <= 1e-12 (FP64) and <= 1e-6 (FP32),
computed in FP64 by the oracle; forward differences to the oracle's
LAPACK-style solve <= 1e-11 (FP64) / 1e-3 (FP32) relative to max|x| in the
median over systems (random U[-1,1] systems reach condition numbers ~1e6).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tridiagonalsolver_gb300 import inputs

pytestmark = pytest.mark.gpu

ETA = {np.float64: 1e-12, np.float32: 1e-6}


def _rel(x, xr):
    return np.max(np.abs(x - xr), axis=1) / np.maximum(np.max(np.abs(xr), axis=1), 1e-300)


def _solve(cuda, arrs, dt, n):
    import tridiagonalsolver_gb300 as T

    batch = arrs[0].shape[0]
    ts = [cuda.from_numpy(np.ascontiguousarray(v.astype(dt))).cuda() for v in arrs]
    info = cuda.full((batch,), -7, dtype=cuda.int32, device="cuda")
    x = T.pge(*ts, n, info=info)
    cuda.cuda.synchronize()
    return x.double().cpu().numpy().reshape(batch, n), info.cpu().numpy()


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("n,batch", [(65, 9), (100, 33), (128, 5), (129, 40), (255, 7), (256, 16), (257, 16),
                                     (1000, 37), (2048, 8), (4095, 8), (4096, 24), (4480, 6)])
def test_pge_matches_oracle(cuda, dt, n, batch):
    a, b, c, d = inputs.nondominant(n, batch, seed=3 * n + batch)
    x, info = _solve(cuda, (a, b, c, d), dt, n)
    assert (info == 0).all()
    a_, b_, c_, d_ = (v.astype(dt).astype(np.float64) for v in (a, b, c, d))
    _, worst = O.backward_error(a_, b_, c_, d_, x, n)
    assert worst <= ETA[dt]
    xo = O.gtsv(a_, b_, c_, d_, n).reshape(batch, n)
    assert np.median(_rel(x, xo)) <= (1e-11 if dt == np.float64 else 1e-3)


@pytest.mark.parametrize("n,batch", [(6000, 4), (8192, 6), (8960, 2)])
def test_pge_fp32_long(cuda, n, batch):
    a, b, c, d = inputs.nondominant(n, batch, seed=n)
    x, info = _solve(cuda, (a, b, c, d), np.float32, n)
    assert (info == 0).all()
    _, worst = O.backward_error(*(v.astype(np.float32).astype(np.float64) for v in (a, b, c, d)), x, n)
    assert worst <= 1e-6


def test_pge_dominant_forward_error(cuda):
    n, batch = 4096, 16
    a, b, c, d = inputs.dominant(n, batch, seed=5)
    x, info = _solve(cuda, (a, b, c, d), np.float64, n)
    xo = O.gtsv(a, b, c, d, n).reshape(batch, n)
    assert np.max(_rel(x, xo)) <= 1e-14


def test_pge_singular_interior_block_falls_back(cuda):
    """Row 32 (first interior row of partition 1 for n = 4096, 128
    partitions) has a zero diagonal and superdiagonal: that interior block is
    singular, the matrix is not."""
    n, batch = 4096, 4
    a, b, c, d = inputs.nondominant(n, batch, seed=11)
    for j in (1, 3):
        b[j, 32] = 0.0
        c[j, 32] = 0.0
        a[j, 32] = 1.0
    import tridiagonalsolver_gb300 as T

    T.lib().tridiag_partition_fallbacks(1)
    x, info = _solve(cuda, (a, b, c, d), np.float64, n)
    assert T.lib().tridiag_partition_fallbacks(1) >= 2
    assert (info == 0).all()
    _, worst = O.backward_error(a, b, c, d, x, n)
    assert worst <= 1e-12


def test_pge_singular_matrix_info(cuda):
    """A zero row makes the matrix singular: info is LAPACK's k+1."""
    from scipy.linalg import lapack

    n, batch = 1000, 3
    a, b, c, d = inputs.nondominant(n, batch, seed=12)
    a[1, 500] = b[1, 500] = c[1, 500] = 0.0
    _, info = _solve(cuda, (a, b, c, d), np.float64, n)
    want = lapack.dgtsv(a[1, 1:].copy(), b[1].copy(), c[1, :-1].copy(), d[1].copy())[4]
    assert info[0] == 0 and info[2] == 0
    assert info[1] == want and want > 0


def test_pge_bench_shape_fp64(cuda):
    """FP64, n = 4096, 4096 non-dominant systems (the pivoted benchmark
    part): all info 0 and 64 sampled systems within the FP64 bar."""
    import tridiagonalsolver_gb300 as T

    torch = cuda
    n, batch = 4096, 4096
    g = torch.Generator(device="cuda")
    g.manual_seed(77)
    a, b, c, d = (torch.rand((batch, n), dtype=torch.float64, device="cuda", generator=g) * 2 - 1 for _ in range(4))
    info = torch.full((batch,), -7, dtype=torch.int32, device="cuda")
    T.partition_path_counts(reset=True)
    x = T.gtsv(a, b, c, d, n, info=info)  # no pivot record requested: the partitioned solve
    assert int((info != 0).sum()) == 0
    paths = T.partition_path_counts(reset=True)
    fb = paths["fallbacks"]
    print(f"partitioned solve of {batch} systems: {paths}")
    assert fb <= batch // 256  # the fast path serves (nearly) every system
    assert T.lib().tridiag_partition_fallbacks(0) == 0  # cleared with the path counts
    assert paths["refinement_passes"] <= paths["exact_checks"] * 2
    idx = torch.arange(0, batch, batch // 64, device="cuda")
    host = [t.index_select(0, idx).cpu().numpy() for t in (a, b, c, d, x)]
    host[0][:, 0] = 0.0
    host[2][:, -1] = 0.0
    _, worst = O.backward_error(*host, n)
    assert worst <= 1e-12


def test_pge_persistent_ring_rare_paths(cuda):
    """FP64 n = 4096 (the TMA-staged persistent kernel) with three systems
    per CTA.  Singular interior blocks are planted in systems that a CTA
    solves first, second (right after another planted one) and last: those
    take the refinement passes, whose copy of x borrows the buffer holding the
    next system's first half, then the sequential solve.  Every system must
    still match the oracle, i.e. no system sees another's rows."""
    import tridiagonalsolver_gb300 as T

    torch = cuda
    n = 4096
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    batch = 3 * sms
    a, b, c, d = inputs.nondominant(n, batch, seed=21)
    planted = (3, 3 + sms, 7 + sms, 9 + 2 * sms, 2 * sms + sms - 1)
    for j in planted:
        b[j, 32] = 0.0
        c[j, 32] = 0.0
        a[j, 32] = 1.0
    T.lib().tridiag_partition_fallbacks(1)
    x, info = _solve(cuda, (a, b, c, d), np.float64, n)
    assert T.lib().tridiag_partition_fallbacks(1) >= len(planted)
    assert (info == 0).all()
    _, worst = O.backward_error(a, b, c, d, x, n)
    assert worst <= 1e-12
    xo = O.gtsv(a, b, c, d, n).reshape(batch, n)
    assert np.median(_rel(x, xo)) <= 1e-11
    # the same batch again: the kernel's results do not depend on the run
    x2, _ = _solve(cuda, (a, b, c, d), np.float64, n)
    assert np.array_equal(x, x2)


def _ppt_rows(torch, n, batch):
    """Partition length of the thread-per-partition solve (ppt.cu: about four
    warps per SM sub-partition, a multiple of 32 rows, at most 64 partitions)."""
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    groups = (batch + 31) // 32
    P = min(max((16 * sms + groups // 2) // groups, 3), 64)
    return (-(-n // P) + 31) // 32 * 32


def _gtsv_many(torch, arrs, n):
    import tridiagonalsolver_gb300 as T

    batch = arrs[0].shape[0]
    a, b, c, d = (torch.from_numpy(np.ascontiguousarray(v)).cuda() for v in arrs)
    info = torch.full((batch,), -7, dtype=torch.int32, device="cuda")
    T.ppt_counts(reset=True)
    x = T.gtsv(a, b, c, d, n, info=info)  # workspace of tridiag_gtsv_workspace_size() bytes
    counts = T.ppt_counts(reset=True)
    return x.cpu().numpy(), info.cpu().numpy(), counts


@pytest.mark.parametrize("n,batch", [(6144, 1024), (7001, 1100), (8192, 1024), (16384, 1024)])
def test_ppt_matches_oracle(cuda, n, batch):
    """Many contiguous FP64 systems longer than one CTA's shared memory holds:
    the thread-per-partition pivoted solve serves them (its counters say so)
    and every system meets the FP64 bar and agrees with the oracle's
    partial-pivoting solve."""
    a, b, c, d = inputs.nondominant(n, batch, seed=7 * n + batch)
    x, info, counts = _gtsv_many(cuda, (a, b, c, d), n)
    assert (info == 0).all()
    assert counts["accepted"] + counts["listed"] == batch
    assert counts["listed"] <= batch // 16
    _, worst = O.backward_error(a, b, c, d, x, n)
    assert worst <= 1e-12
    xo = O.gtsv(a, b, c, d, n).reshape(batch, n)
    assert np.median(_rel(x.reshape(batch, n), xo)) <= 1e-11


def test_ppt_singular_partition_falls_back(cuda):
    """A zero diagonal and superdiagonal in the first interior row of
    partition 1 makes that partition's block singular (the matrix is not):
    those systems miss the acceptance test and the partitioned solve (here
    in clusters) takes them."""
    n, batch = 6144, 1024
    L = _ppt_rows(cuda, n, batch)
    a, b, c, d = inputs.nondominant(n, batch, seed=31)
    planted = (0, 5, 1000, batch - 1)
    for j in planted:
        b[j, L] = 0.0
        c[j, L] = 0.0
        a[j, L] = 1.0
    x, info, counts = _gtsv_many(cuda, (a, b, c, d), n)
    assert counts["listed"] >= len(planted)
    assert counts["accepted"] + counts["listed"] == batch
    assert (info == 0).all()
    _, worst = O.backward_error(a, b, c, d, x, n)
    assert worst <= 1e-12


def test_ppt_not_for_one_cta_sizes(cuda):
    """At 4096 rows the persistent one-CTA solve keeps the batch (the
    thread-per-partition solve would be no faster there, in five launches)."""
    import tridiagonalsolver_gb300 as T

    a, b, c, d = inputs.nondominant(4096, 1024, seed=43)
    x, info, counts = _gtsv_many(cuda, (a, b, c, d), 4096)
    assert counts == {"accepted": 0, "listed": 0}
    assert (info == 0).all()


def test_ppt_out_of_place(cuda):
    """solve_out with TRIDIAG_ALGO_GTSV (the benchmark's call): the same
    solve out of place -- d untouched, the listed systems solved again from
    it -- including systems planted to miss the acceptance test."""
    import tridiagonalsolver_gb300 as T

    torch = cuda
    n, batch = 6144, 1024
    L = _ppt_rows(torch, n, batch)
    a, b, c, d = inputs.nondominant(n, batch, seed=41)
    for j in (2, 700):
        b[j, L] = 0.0
        c[j, L] = 0.0
        a[j, L] = 1.0
    ta, tb, tc, td = (torch.from_numpy(np.ascontiguousarray(v)).cuda() for v in (a, b, c, d))
    x = torch.empty_like(td)
    work = T.solve_out_workspace(ta, n, "gtsv")
    T.ppt_counts(reset=True)
    T.solve_out(ta, tb, tc, td, n, algo="gtsv", out=x, work=work)
    counts = T.ppt_counts(reset=True)
    assert counts["accepted"] + counts["listed"] == batch and counts["listed"] >= 2
    assert np.array_equal(td.cpu().numpy(), d)
    xh = x.cpu().numpy()
    _, worst = O.backward_error(a, b, c, d, xh, n)
    assert worst <= 1e-12
    # in place (gtsv) gives the same bits
    x2, _, _ = _gtsv_many(torch, (a, b, c, d), n)
    assert np.array_equal(x2, xh)


@pytest.mark.parametrize("n,batch,planted", [(4096, 1024, ()), (3000, 2048, (1, 777, 2047))])
def test_ppt_interleaved(cuda, n, batch, planted):
    """Batch-interleaved FP64 systems (layout 2): the thread-per-partition
    solve serves them with every access coalesced; planted singular partition
    blocks take the masked sequential solve.  Every system meets the FP64 bar
    and agrees with the oracle."""
    import tridiagonalsolver_gb300 as T

    torch = cuda
    L = _ppt_rows(torch, n, batch)
    a, b, c, d = inputs.nondominant(n, batch, seed=n + batch)
    for j in planted:
        b[j, L] = 0.0
        c[j, L] = 0.0
        a[j, L] = 1.0
    ti = [torch.from_numpy(np.ascontiguousarray(v)).cuda() for v in inputs.to_interleaved(a, b, c, d)]
    info = torch.full((batch,), -7, dtype=torch.int32, device="cuda")
    T.ppt_counts(reset=True)
    x = T.gtsv(*ti, n, layout="interleaved", info=info)
    counts = T.ppt_counts(reset=True)
    assert counts["accepted"] + counts["listed"] == batch
    assert counts["listed"] >= len(planted) and counts["listed"] <= len(planted) + batch // 64
    assert (info.cpu().numpy() == 0).all()
    xh = x.cpu().numpy().T.copy()
    _, worst = O.backward_error(a, b, c, d, xh, n)
    assert worst <= 1e-12
    xo = O.gtsv(a, b, c, d, n).reshape(batch, n)
    assert np.median(_rel(xh, xo)) <= 1e-11


def test_ppt_long_systems_fp64(cuda):
    """FP64 8192 x 4096 non-dominant through gtsv: the thread-per-partition
    solve serves it, (nearly) every system is accepted there, and 64 sampled
    systems meet the FP64 bar."""
    import tridiagonalsolver_gb300 as T

    torch = cuda
    n, batch = 8192, 4096
    g = torch.Generator(device="cuda")
    g.manual_seed(77)
    a, b, c, d = (torch.rand((batch, n), dtype=torch.float64, device="cuda", generator=g) * 2 - 1 for _ in range(4))
    d0 = d.clone()
    info = torch.full((batch,), -7, dtype=torch.int32, device="cuda")
    T.ppt_counts(reset=True)
    x = T.gtsv(a, b, c, d, n, info=info)
    counts = T.ppt_counts(reset=True)
    print(f"thread-per-partition solve of {batch} systems: {counts}")
    assert counts["accepted"] + counts["listed"] == batch
    assert counts["listed"] <= batch // 256
    assert int((info != 0).sum()) == 0
    idx = torch.arange(0, batch, batch // 64, device="cuda")
    host = [t.index_select(0, idx).cpu().numpy() for t in (a, b, c, d0, x)]
    host[0][:, 0] = 0.0
    host[2][:, -1] = 0.0
    _, worst = O.backward_error(*host, n)
    assert worst <= 1e-12
    xo = O.gtsv(*host[:4], n).reshape(-1, n)
    assert np.median(_rel(host[4], xo)) <= 1e-11


@pytest.mark.parametrize("name,dt,n", [("WM5_reg_double", np.float64, 4096), ("WM4_shmem_single", np.float32, 3000)])
def test_reference_wm_names_long_systems(cuda, name, dt, n):
    """The reference's WM entry points on systems beyond one warp use the
    partitioned solve (in place, d <- x)."""
    import tridiagonalsolver_gb300 as T

    batch = 8
    a, b, c, d = inputs.dominant(n, batch, seed=n)
    ts = [cuda.from_numpy(v.astype(dt)).cuda() for v in (a, b, c, d)]
    T.reference_call(name, *ts, n)
    x = ts[3].double().cpu().numpy().reshape(batch, n)
    _, worst = O.backward_error(*(v.astype(dt).astype(np.float64) for v in (a, b, c, d)), x, n)
    assert worst <= ETA[dt]


def test_pge_unsupported_sizes(cuda):
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import TridiagError

    for dt, n in ((cuda.float64, 1), (cuda.float64, 64), (cuda.float64, 30000), (cuda.float32, 70000)):
        t = cuda.ones(n * 2, dtype=dt, device="cuda")
        with pytest.raises(TridiagError):
            T.pge(t, t, t, t, n)


def test_bplg_packed_long(cuda):
    """Packed layout (BPLG entry point) through the partitioned solve."""
    import tridiagonalsolver_gb300 as T

    n, batch = 2048, 6
    a, b, c, d = inputs.dominant(n, batch, seed=4)
    packed = cuda.from_numpy(inputs.to_packed(a, b, c, d).astype(np.float32)).cuda()
    T.lib().BPLG_WM(packed.data_ptr(), packed.data_ptr() + 4 * n, packed.data_ptr() + 8 * n,
                    packed.data_ptr() + 12 * n, n, batch)
    assert T.last_status() == 0
    x = packed.double().cpu().numpy().reshape(batch, 4, n)[:, 3, :]
    _, worst = O.backward_error(*(v.astype(np.float32).astype(np.float64) for v in (a, b, c, d)), x, n)
    assert worst <= 1e-6


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("n,batch,shift", [(4096, 9, (0, 0, 0, 0, 1)), (1000, 7, (1, 2, 3, 1, 2)),
                                           (3001, 5, (3, 0, 1, 2, 0)), (20000, 3, (0, 1, 0, 3, 2))])
def test_pge_any_alignment(cuda, dt, n, batch, shift):
    """Arrays at element offsets that put each one in its own 16-byte phase
    (the bulk staging copies each array's aligned rows and the rest
    element-wise; x in a phase other than d's leaves element-wise): the same
    result as the aligned call, bit for bit, and the oracle's bar.  n = 20000
    runs the cluster version.  At n = 4096 FP64 the aligned call runs the
    TMA-staged kernel (32-row partitions) and the shifted x sends the call to
    the dense layout (33-row partitions): the same bar, other roundings."""
    import tridiagonalsolver_gb300 as T

    torch = cuda
    a, b, c, d = inputs.nondominant(n, batch, seed=n + 5)
    td = torch.float64 if dt == np.float64 else torch.float32
    aligned = [torch.from_numpy(np.ascontiguousarray(v.astype(dt))).cuda() for v in (a, b, c, d)]
    x0 = T.pge(*aligned, n)
    shifted = []
    for v, k in zip(aligned, shift[:4]):
        buf = torch.empty(v.numel() + 8, dtype=td, device="cuda")
        buf[k:k + v.numel()].copy_(v.reshape(-1))
        shifted.append(buf[k:k + v.numel()])
    xb = torch.empty(batch * n + 8, dtype=td, device="cuda")
    x1 = xb[shift[4]:shift[4] + batch * n]
    # through the C ABI: the Python front end copies inputs at odd offsets
    p = "double" if dt == np.float64 else "single"
    st = getattr(T.lib(), f"tridiag_pge_{p}")(0, *(v.data_ptr() for v in shifted), x1.data_ptr(), None, n, batch,
                                            torch.cuda.current_stream().cuda_stream)
    assert st == 0
    torch.cuda.synchronize()
    if dt == np.float64 and n == 4096:
        assert float((x0.reshape(-1) - x1).abs().max() / x0.abs().max()) <= 1e-10
    else:
        assert torch.equal(x0.reshape(-1), x1)
    a_, b_, c_, d_ = (v.astype(dt).astype(np.float64) for v in (a, b, c, d))
    _, worst = O.backward_error(a_, b_, c_, d_, x1.double().cpu().numpy(), n)
    assert worst <= ETA[dt]
