"""The tcgen05 tensor-core GEMM building block (BF16 operands via TMA, FP32
accumulation in tensor memory) against an FP64 product of the same BF16
values.  Tolerance: FP32 accumulation over K, 1e-5 relative to the sum of
absolute products."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def to_bf16_bits(x):
    """float32 -> bfloat16 bit patterns, round to nearest even."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    rounded = b + 0x7FFF + ((b >> 16) & 1)
    return (rounded >> 16).astype(np.uint16)


def bf16_bits_to_f64(h):
    return (h.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def run(lib, m, n, k, J, seed):
    rng = np.random.default_rng(seed)
    A = to_bf16_bits(rng.standard_normal((m, k)).astype(np.float32))
    Bs = [to_bf16_bits(rng.standard_normal((n, k)).astype(np.float32)) for _ in range(J)]
    Cs = [rng.standard_normal((m, n)).astype(np.float32) for _ in range(J)]
    dev = []

    def up(arr):
        p = lib.peec_gb300_device_alloc(arr.nbytes)
        assert lib.peec_gb300_copy_to_device(p, arr.ctypes.data, arr.nbytes) == 0
        dev.append(p)
        return p
    dA = up(A)
    dB = [up(b) for b in Bs]
    dC = [up(c) for c in Cs]
    s = lib.peec_gb300_tc_gemm(dA, dB[0], dB[-1], dC[0], dC[-1], m, n, k, n, J)
    outs = []
    for j in range(J):
        o = np.zeros((m, n), dtype=np.float32)
        lib.peec_gb300_copy_to_host(o.ctypes.data, dC[j], o.nbytes)
        outs.append(o)
    for p in dev:
        lib.peec_gb300_device_free(p)
    Af = bf16_bits_to_f64(A)
    for j in range(J):
        Bf = bf16_bits_to_f64(Bs[j])
        ref = Cs[j].astype(np.float64) - Af @ Bf.T
        scale = np.abs(Cs[j]) + np.abs(Af) @ np.abs(Bf).T
        err = np.max(np.abs(outs[j] - ref) / scale)
        assert err < 1e-5, (m, n, k, J, j, err)
    return s


@pytest.mark.parametrize("m,n,k,J", [(128, 128, 64, 1), (256, 384, 192, 1), (200, 130, 128, 1),
                                     (384, 256, 384, 2), (131, 77, 64, 2), (1024, 1024, 384, 2)])
def test_tc_gemm_matches_fp64(gpu_lib, m, n, k, J):
    assert run(gpu_lib, m, n, k, J, seed=m + n + k + J) == 0


def test_tc_gemm_rejects_bad_k(gpu_lib):
    assert gpu_lib.peec_gb300_tc_gemm(1, 1, 1, 1, 1, 128, 128, 100, 128, 1) == -1


def run_cplx(lib, m, n, k, row0, col0, ldc, rows, seed):
    """C (rows x ldc interleaved complex FP32) block [row0.., col0..] -= A Br^T + j A Bi^T;
    everything outside the block must be untouched bit for bit."""
    rng = np.random.default_rng(seed)
    A = to_bf16_bits(rng.standard_normal((m, k)).astype(np.float32))
    Br = to_bf16_bits(rng.standard_normal((n, k)).astype(np.float32))
    Bi = to_bf16_bits(rng.standard_normal((n, k)).astype(np.float32))
    C0 = rng.standard_normal((rows, 2 * ldc)).astype(np.float32)
    dev = []

    def up(arr):
        p = lib.peec_gb300_device_alloc(arr.nbytes)
        assert lib.peec_gb300_copy_to_device(p, arr.ctypes.data, arr.nbytes) == 0
        dev.append(p)
        return p
    dA, dBr, dBi, dC = up(A), up(Br), up(Bi), up(C0)
    s = lib.peec_gb300_tc_gemm_cplx(dA, dBr, dBi, dC, m, n, k, row0, col0, ldc)
    out = np.zeros_like(C0)
    lib.peec_gb300_copy_to_host(out.ctypes.data, dC, out.nbytes)
    for p in dev:
        lib.peec_gb300_device_free(p)
    assert s == 0
    Af, Brf, Bif = bf16_bits_to_f64(A), bf16_bits_to_f64(Br), bf16_bits_to_f64(Bi)
    blk = (slice(row0, row0 + m), slice(2 * col0, 2 * (col0 + n)))
    ref = C0.astype(np.float64).copy()
    ref[blk[0], blk[1].start:blk[1].stop:2] -= Af @ Brf.T
    ref[blk[0], blk[1].start + 1:blk[1].stop:2] -= Af @ Bif.T
    scale = np.abs(C0).astype(np.float64)
    scale[blk[0], blk[1].start:blk[1].stop:2] += np.abs(Af) @ np.abs(Brf).T
    scale[blk[0], blk[1].start + 1:blk[1].stop:2] += np.abs(Af) @ np.abs(Bif).T
    err = np.max(np.abs(out - ref) / scale)
    assert err < 1e-5, (m, n, k, err)
    mask = np.ones(C0.shape, dtype=bool)
    mask[blk] = False
    assert np.array_equal(out[mask], C0[mask])


# (m, n, k, row0, col0, ldc, rows): even ldc and an aligned block take the
# persistent kernel (128-column tiles, or 64-column tiles for K <= 192 and
# for K <= 384 with at most 256 columns;
# several tiles per CTA at the larger sizes, ragged edges); odd ldc takes
# the one-tile-per-CTA kernels.
@pytest.mark.parametrize("m,n,k,row0,col0,ldc,rows", [
    (128, 128, 384, 0, 0, 128, 128), (300, 260, 1536, 5, 6, 600, 320), (1000, 700, 768, 2, 4, 800, 1010),
    (4000, 2600, 256, 32, 64, 2700, 4040), (200, 150, 384, 1, 3, 301, 210), (500, 100, 192, 0, 32, 200, 510),
    (8000, 224, 192, 40, 64, 600, 8040), (300, 90, 192, 1, 3, 301, 310), (2000, 224, 384, 8, 32, 400, 2040)])
def test_tc_gemm_cplx_block(gpu_lib, m, n, k, row0, col0, ldc, rows):
    run_cplx(gpu_lib, m, n, k, row0, col0, ldc, rows, seed=m + n + k)
