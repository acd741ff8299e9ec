"""FFT (cufftExecC2C replacement) and FP32 Hermitian X-engine
(cublasCgemmBatched replacement) against the FP64 oracle."""
import numpy as np
import pytest
import torch

from conftest import rel_fro

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("n", [2, 4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096, 8192, 16384])
def test_fft_vs_oracle(mdt, cuda, oracle, n):
    rows = max(3, 4096 // n)
    rng = np.random.default_rng(n)
    x = (rng.standard_normal((rows, n)) + 1j * rng.standard_normal((rows, n))).astype(np.complex64)
    ref = oracle.fft_rows(x.astype(np.complex128), n).reshape(rows, n)
    xd = dev(x)
    out = torch.empty_like(xd)
    mdt.fft_c2c(xd, out, rows, n, -1)
    torch.cuda.synchronize()
    y = out.cpu().numpy()
    err = np.linalg.norm(y - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert err.max() < 3e-7 * max(1, np.log2(n)), err.max()
    # in place gives the same bits
    mdt.fft_c2c(xd, xd, rows, n, -1)
    torch.cuda.synchronize()
    assert np.array_equal(xd.cpu().numpy().view(np.uint32), y.view(np.uint32))


def test_fft_inverse_roundtrip_and_shim(mdt, cuda):
    n, rows = 1024, 64
    rng = np.random.default_rng(1)
    x = (rng.standard_normal((rows, n)) + 1j * rng.standard_normal((rows, n))).astype(np.complex64)
    xd = dev(x)
    plan = mdt.cufftPlan1d(n, mdt.CUFFT_C2C, rows)
    mdt.cufftSetStream(plan, torch.cuda.current_stream())
    mdt.cufftExecC2C(plan, xd, xd, mdt.CUFFT_FORWARD)
    mdt.cufftExecC2C(plan, xd, xd, mdt.CUFFT_INVERSE)
    torch.cuda.synchronize()
    np.testing.assert_allclose(xd.cpu().numpy() / n, x, rtol=0, atol=1e-5)
    mdt.cufftDestroy(plan)
    with pytest.raises(mdt.MdtError) as e:
        mdt.cufftPlan1d(1000, mdt.CUFFT_C2C, 1)
    assert e.value.code == 0x8  # CUFFT_INVALID_SIZE
    with pytest.raises(mdt.MdtError) as e:
        mdt.cufftExecC2C(plan, xd, xd, mdt.CUFFT_FORWARD)
    assert e.value.code == 0x1  # CUFFT_INVALID_PLAN
    assert mdt.cufftGetVersion() == 1000


# (NE <= 60 runs two channels per block: odd channel counts leave a lone last channel;
#  NE = 61..64 is a single diagonal super-tile that does not fit twice in a block)
@pytest.mark.parametrize("ne,nch,nsp", [(3, 4, 2), (10, 8, 1000), (40, 6, 333), (64, 3, 64),
                                        (65, 2, 100), (130, 2, 70), (256, 2, 96), (60, 5, 40),
                                        (61, 3, 40), (7, 1, 17)])
def test_xengine_f32_vs_oracle(mdt, cuda, oracle, ne, nch, nsp):
    rng = np.random.default_rng(ne * 1000 + nsp)
    X = (rng.standard_normal((nch, nsp, ne)) + 1j * rng.standard_normal((nch, nsp, ne))
         ).astype(np.complex64)
    ref = oracle.xengine(X.astype(np.complex128), ne, nch, nsp, 1.0 / nsp)
    V = torch.full((nch, ne, ne), float("nan"), dtype=torch.complex64, device=cuda)
    mdt.xengine_f32(ne, nch, nsp, dev(X), ne, nsp * ne, 1.0 / nsp, V)
    torch.cuda.synchronize()
    v = V.cpu().numpy()
    assert rel_fro(v, ref) < 1e-6
    # exact Hermitian mirror, real diagonal
    assert np.array_equal(v, np.conj(np.transpose(v, (0, 2, 1))))
    assert np.all(np.diagonal(v, axis1=1, axis2=2).imag == 0)


def _ptr_array(base, stride_elems, count):
    return torch.tensor([base.data_ptr() + i * stride_elems * 8 for i in range(count)],
                        dtype=torch.int64, device=base.device)


def test_cublas_shim_hermitian_reference_call(mdt, cuda, oracle):
    # the reference's exact call: (N, C, NE, NE, Nsp, 1/Nsp, A=B=XinPtr, beta=0)
    ne, nch, nsp = 12, 16, 50
    rng = np.random.default_rng(2)
    X = (rng.standard_normal((nch, nsp, ne)) + 1j * rng.standard_normal((nch, nsp, ne))
         ).astype(np.complex64)
    Xd = dev(X)
    V = torch.full((nch, ne, ne), float("nan"), dtype=torch.complex64, device=cuda)
    A = _ptr_array(Xd, ne * nsp, nch)
    C = _ptr_array(V, ne * ne, nch)
    h = mdt.cublasCreate()
    mdt.cublasSetStream(h, torch.cuda.current_stream())
    mdt.cublasCgemmBatched(h, mdt.CUBLAS_OP_N, mdt.CUBLAS_OP_C, ne, ne, nsp, 1.0 / nsp, A, ne, A,
                           ne, 0.0, C, ne, nch)
    torch.cuda.synchronize()
    ref = oracle.xengine(X.astype(np.complex128), ne, nch, nsp, 1.0 / nsp)
    assert rel_fro(V.cpu().numpy(), ref) < 1e-6
    # complex alpha and nonzero beta through the same path
    V0 = V.clone()
    mdt.cublasCgemmBatched(h, mdt.CUBLAS_OP_N, mdt.CUBLAS_OP_C, ne, ne, nsp, 0.5 - 0.25j, A, ne, A,
                           ne, 2.0 + 1.0j, C, ne, nch)
    torch.cuda.synchronize()
    want = (0.5 - 0.25j) * ref * nsp + (2.0 + 1.0j) * V0.cpu().numpy().astype(np.complex128)
    assert rel_fro(V.cpu().numpy(), want) < 1e-6
    mdt.cublasDestroy(h)


@pytest.mark.parametrize("ta,tb", [(0, 0), (0, 1), (1, 0), (2, 2), (1, 2)])
def test_cublas_shim_general(mdt, cuda, ta, tb):
    m, n, k, batch = 7, 5, 9, 3
    rng = np.random.default_rng(ta * 3 + tb)

    def mat(r, c):
        return (rng.standard_normal((batch, r, c)) + 1j * rng.standard_normal((batch, r, c))
                ).astype(np.complex64)

    def op(M, t):
        return M if t == 0 else (np.transpose(M, (0, 2, 1)) if t == 1
                                 else np.conj(np.transpose(M, (0, 2, 1))))

    A = mat(m, k) if ta == 0 else mat(k, m)  # column-major storage = numpy transpose
    B = mat(k, n) if tb == 0 else mat(n, k)
    Cm = mat(m, n)
    # store column-major: element (i, j) at i + j*ld  -> numpy array [j][i]
    Ad = dev(np.ascontiguousarray(np.transpose(A, (0, 2, 1))))
    Bd = dev(np.ascontiguousarray(np.transpose(B, (0, 2, 1))))
    Cd = dev(np.ascontiguousarray(np.transpose(Cm, (0, 2, 1))))
    lda, ldb = A.shape[1], B.shape[1]
    h = mdt.cublasCreate()
    mdt.cublasCgemmBatched(h, ta, tb, m, n, k, 1.5 + 0.5j,
                           _ptr_array(Ad, A.shape[1] * A.shape[2], batch), lda,
                           _ptr_array(Bd, B.shape[1] * B.shape[2], batch), ldb, -1.0,
                           _ptr_array(Cd, m * n, batch), m, batch)
    torch.cuda.synchronize()
    ref = (1.5 + 0.5j) * (op(A.astype(np.complex128), ta) @ op(B.astype(np.complex128), tb)) - Cm
    got = np.transpose(Cd.cpu().numpy(), (0, 2, 1))
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-4)
    mdt.cublasDestroy(h)
