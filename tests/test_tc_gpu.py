"""GPU parity of the tcgen05 tensor-core trailing update (BF16 and split-BF16)
against an FP64 host reference of the same products, through the C-ABI."""
import numpy as np
import pytest

from starpu_gb300 import DeviceBuffer
from starpu_gb300.native import check

pytestmark = pytest.mark.gpu


def bf16_bits(x):
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return ((u + ((u >> 16) & 1) + 0x7FFF) >> 16).astype(np.uint16)


def bf16_val(bits):
    return (bits.astype(np.uint32) << 16).view(np.float32)


def kmajor(bits, ldk):
    m, k = bits.shape
    out = np.zeros((m, ldk), dtype=np.uint16)
    out[:, :k] = bits
    return out


def zeros_err():
    e = DeviceBuffer(4)
    e.upload(np.zeros(1, np.int32))
    return e


@pytest.mark.parametrize("m,n,k", [(128, 256, 64), (300, 520, 200), (1000, 300, 1024), (64, 17, 8)])
def test_tc_update_bf16_rect(gpu, m, n, k):
    rng = np.random.default_rng(m * 31 + n * 7 + k)
    A = bf16_bits(rng.standard_normal((m, k)))
    B = bf16_bits(rng.standard_normal((n, k)))
    Cm = rng.standard_normal((m, n)).astype(np.float32)
    ldk = (k + 63) // 64 * 64
    dA = DeviceBuffer.from_array(np.ascontiguousarray(kmajor(A, ldk)).ravel())
    dB = DeviceBuffer.from_array(np.ascontiguousarray(kmajor(B, ldk)).ravel())
    dC = DeviceBuffer.from_array(Cm)
    err = zeros_err()
    check(gpu.starpu_gb300_tc_update(None, m, n, k, dA.ptr, None, ldk, dB.ptr, None, ldk, 1, 0, dC.ptr, m, err.ptr))
    out = dC.download((m, n), np.float32)
    assert err.download((1,), np.int32)[0] == 0
    ref = Cm.astype(np.float64) - bf16_val(A).astype(np.float64) @ bf16_val(B).astype(np.float64).T
    assert np.max(np.abs(out - ref)) <= 2e-6 * np.sqrt(k) * max(1.0, np.max(np.abs(ref)))


@pytest.mark.parametrize("m,k", [(256, 64), (513, 384), (2048, 1024)])
def test_tc_update_bf16_lower_syrk(gpu, m, k):
    rng = np.random.default_rng(m + k)
    A = bf16_bits(rng.standard_normal((m, k)))
    Cm = rng.standard_normal((m, m)).astype(np.float32)
    ldk = (k + 63) // 64 * 64
    dA = DeviceBuffer.from_array(np.ascontiguousarray(kmajor(A, ldk)).ravel())
    dC = DeviceBuffer.from_array(Cm)
    err = zeros_err()
    check(gpu.starpu_gb300_tc_update(None, m, m, k, dA.ptr, None, ldk, dA.ptr, None, ldk, 1, 1, dC.ptr, m, err.ptr))
    out = dC.download((m, m), np.float32)
    assert err.download((1,), np.int32)[0] == 0
    Af = bf16_val(A).astype(np.float64)
    ref = Cm.astype(np.float64) - Af @ Af.T
    lo = np.tril_indices(m)
    assert np.max(np.abs(out[lo] - ref[lo])) <= 2e-6 * np.sqrt(k) * max(1.0, np.max(np.abs(ref)))
    upi = np.triu_indices(m, 1)
    assert np.array_equal(out[upi], Cm[upi])


@pytest.mark.parametrize("m,k", [(384, 256), (1100, 512)])
def test_split_bf16_x3_accuracy(gpu, m, k):
    """split-BF16 (3 products) carries ~16 bits: far closer to the FP64 product
    than plain BF16, with the same tensor-core kernel."""
    rng = np.random.default_rng(5)
    P = rng.standard_normal((m, k)).astype(np.float32)
    Cm = np.zeros((m, m), dtype=np.float32, order="F")
    ldk = (k + 63) // 64 * 64
    dP = DeviceBuffer.from_array(P)
    hi, lo = DeviceBuffer(m * ldk * 2), DeviceBuffer(m * ldk * 2)
    check(gpu.starpu_gb300_split_bf16(None, m, k, dP.ptr, m, hi.ptr, lo.ptr, ldk))
    h = hi.download((m * ldk,), np.uint16).reshape(m, ldk)
    np.testing.assert_array_equal(h[:, :k], bf16_bits(P))
    assert not h[:, k:].any()
    ref = -(P.astype(np.float64) @ P.astype(np.float64).T)
    errs = {}
    for nterms in (1, 3):
        dC = DeviceBuffer.from_array(Cm)
        err = zeros_err()
        check(gpu.starpu_gb300_tc_update(None, m, m, k, hi.ptr, lo.ptr, ldk, hi.ptr, lo.ptr, ldk, nterms, 1, dC.ptr, m,
                                         err.ptr))
        out = dC.download((m, m), np.float32)
        assert err.download((1,), np.int32)[0] == 0
        li = np.tril_indices(m)
        errs[nterms] = np.max(np.abs(out[li] - ref[li])) / np.max(np.abs(ref))
    assert errs[1] < 2e-2
    assert errs[3] < 5e-5
    assert errs[3] < errs[1] / 50


@pytest.mark.parametrize("n,nb,nterms", [(2048, 256, 3), (2048, 512, 1), (1000, 256, 3)])
def test_spotrf_tc_hilbert(gpu, oracle, n, nb, nterms):
    A = oracle.hilbert_f32(n)
    d = DeviceBuffer.from_array(A)
    ws = gpu.starpu_gb300_spotrf_tc_workspace(n, nb)
    W = DeviceBuffer(ws)
    info, err = zeros_err(), zeros_err()
    check(gpu.starpu_gb300_spotrf_tc(None, n, d.ptr, n, nb, nterms, W.ptr, ws, info.ptr, err.ptr))
    L = d.download((n, n), np.float32)
    assert info.download((1,), np.int32)[0] == 0
    assert err.download((1,), np.int32)[0] == 0
    bad, worst = oracle.check_hilbert(L, 1e-4)
    assert bad == 0, worst


def test_spotrf_tc_gram_residual(gpu, oracle):
    n, nb = 1536, 512
    A = oracle.spd_gram(n, 4, 1.0)
    res = {}
    for nterms in (1, 3):
        d = DeviceBuffer.from_array(A.astype(np.float32))
        ws = gpu.starpu_gb300_spotrf_tc_workspace(n, nb)
        W = DeviceBuffer(ws)
        info, err = zeros_err(), zeros_err()
        check(gpu.starpu_gb300_spotrf_tc(None, n, d.ptr, n, nb, nterms, W.ptr, ws, info.ptr, err.ptr))
        L = np.tril(d.download((n, n), np.float32))
        assert info.download((1,), np.int32)[0] == 0
        res[nterms] = oracle.llt_residual(A, L)
    # the factorisation's panels reach the tensor cores as row-scaled FP16
    # splits (~22 bits; the BF16 split measured 3.9e-6 at n = 8192): three
    # products land within a few times the FP32 accumulation error
    assert res[1] < 1e-3
    assert res[3] < 3e-6


@pytest.mark.parametrize("n,nb", [(2000, 1000), (700, 333), (1088, 1024), (130, 64), (1024, 1024)])
def test_spotrf_tc_diagonal_tile_shapes(gpu, oracle, n, nb):
    """The diagonal tile is factored and inverted by one cooperative launch in
    64 x 64 blocks: ragged last blocks (1000 = 15 x 64 + 40, 333), a ragged
    last doubling pair, a 64 tail, a tile with no panel below it.  The factor
    meets the split-BF16 residual bound, the strict upper triangle is never
    written, and no barrier wait runs out."""
    A = oracle.spd_gram(n, 7, 1.0).astype(np.float32)
    A[np.triu_indices(n, 1)] = -3.0  # never read, never written
    d = DeviceBuffer.from_array(A)
    ws = gpu.starpu_gb300_spotrf_tc_workspace(n, nb)
    W = DeviceBuffer(ws)
    info, err = zeros_err(), zeros_err()
    check(gpu.starpu_gb300_spotrf_tc(None, n, d.ptr, n, nb, 3, W.ptr, ws, info.ptr, err.ptr))
    out = d.download((n, n), np.float32)
    assert info.download((1,), np.int32)[0] == 0
    assert err.download((1,), np.int32)[0] == 0
    np.testing.assert_array_equal(out[np.triu_indices(n, 1)], -3.0)
    Af = np.tril(A.astype(np.float64)) + np.tril(A.astype(np.float64), -1).T
    assert oracle.llt_residual(Af, np.tril(out)) < 1e-5


def test_spotrf_tc_reports_the_first_non_positive_pivot(gpu):
    n, nb = 700, 333
    A = np.eye(n, dtype=np.float32) * 2
    A[450, 450] = -1.0  # tile 1 (333..665), 64-block 1 of that tile, row 53 of it
    d = DeviceBuffer.from_array(A)
    ws = gpu.starpu_gb300_spotrf_tc_workspace(n, nb)
    W = DeviceBuffer(ws)
    info, err = zeros_err(), zeros_err()
    check(gpu.starpu_gb300_spotrf_tc(None, n, d.ptr, n, nb, 3, W.ptr, ws, info.ptr, err.ptr))
    assert info.download((1,), np.int32)[0] == 451
    assert err.download((1,), np.int32)[0] == 0

