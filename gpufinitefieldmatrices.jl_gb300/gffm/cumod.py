"""CuModArray / CuModMatrix / CuModVector: the reference's container, on the GB300.

Mirrors src/CuModMatrix/CuModMatrix.jl:42-181: ``data`` is a device buffer
padded by 32 in every dimension (column-major: element (i, j) of the padded
(rows+32) x (cols+32) array), ``size`` is the true size and ``N`` the modulus.
Storage is a torch CUDA tensor (PyTorch is only the allocator and stream
here); every operation calls libgffm through its C ABI.  Method names follow
the reference, with Julia's ``!`` spelled as a trailing underscore
(``mul!`` -> ``mul_``).
"""
import ctypes

import numpy as np
import torch

from ._lib import call

TILE_WIDTH = 32                 # CuModMatrix.jl:2
DEFAULT_TYPE = torch.float32    # CuModMatrix.jl:3


class CuModArraySizeMismatchException(Exception):
    pass


class CuModArrayModulusMismatchException(Exception):
    pass


class CuModMatrixNotSquareException(Exception):
    pass


class CuModMatrixModulusNotPrimeException(Exception):
    pass


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _sfx(dtype):
    if dtype == torch.float64:
        return "f64"
    if dtype == torch.float32:
        return "f32"
    raise TypeError("CuModArray storage must be torch.float32 or torch.float64 (got %s)" % dtype)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class CuModArray:
    """A matrix (D = 2) or vector (D = 1) over Z/N with padded device storage."""

    def __init__(self, data, size, N):
        if N > 2 ** 52:
            raise CuModArrayModulusMismatchException(
                "Modulus %d is bigger than 2^52 = %d, the largest supported modulus" % (N, 2 ** 52))
        self.data = data            # torch tensor, (cols+32, rows+32) for matrices
        self.size = tuple(int(s) for s in size)
        self.N = int(N)

    # -- shape helpers -----------------------------------------------------
    @property
    def ndim(self):
        return len(self.size)

    @property
    def ld(self):
        return self.data.shape[-1]

    @property
    def dtype(self):
        return self.data.dtype

    def rows(self):
        return self.size[0]

    def cols(self):
        return self.size[1] if self.ndim == 2 else 1

    def __len__(self):
        return int(np.prod(self.size))

    @property
    def padded_len(self):
        return self.data.numel()

    def __repr__(self):
        return "%s CuModArray modulo %d:\n%s" % ("x".join(map(str, self.size)), self.N, self.Array())

    # -- host conversion ---------------------------------------------------
    def Array(self):
        """Array(A): the unpadded contents as a numpy array (CuModMatrix.jl:256-261)."""
        h = self.data.detach().cpu().numpy()
        if self.ndim == 1:
            return h[: self.size[0]].copy()
        return h.T[: self.size[0], : self.size[1]].copy()

    def unsafe_Array(self):
        h = self.data.detach().cpu().numpy()
        return h.copy() if self.ndim == 1 else h.T.copy()

    # -- operators (kernel_ops/*.jl) ---------------------------------------
    def __add__(self, other):
        C = similar(self)
        if isinstance(other, CuModArray):
            add_(C, self, other)
        else:
            scalar_add_(C, self, other)
        return C

    __radd__ = __add__

    def __sub__(self, other):
        C = similar(self)
        if isinstance(other, CuModArray):
            sub_(C, self, other)
        else:
            scalar_sub_(C, self, other)
        return C

    def __rsub__(self, s):
        C = similar(self)
        rscalar_sub_(C, self, s)
        return C

    def __neg__(self):
        C = similar(self)
        negate_(C, self)
        return C

    def __mul__(self, other):
        if isinstance(other, CuModArray):
            if self.ndim == 2 and other.ndim == 2:
                C = zeros(self.dtype, self.rows(), other.cols(), self.N)
                mul_(C, self, other)
                return C
            if self.ndim == 2 and other.ndim == 1:
                z = zeros(self.dtype, self.rows(), self.N)
                mul_(z, self, other)
                return z
            raise TypeError("unsupported product")
        C = similar(self)
        scalar_mul_(C, self, other)
        return C

    def __rmul__(self, s):
        return self.__mul__(s)

    def __truediv__(self, s):
        """A / s (div_ops.jl:24-28): A times the reference's mod_inv(s, N)."""
        C = similar(self)
        div_(C, self, s)
        return C

    def __matmul__(self, other):
        return self.__mul__(other)

    def __pow__(self, n):
        """Recursive binary exponentiation (CuModMatrix.jl:307-329)."""
        if self.rows() != self.cols():
            raise CuModMatrixNotSquareException("Matrix must be square for power operation")
        if n == 0:
            return eye(self.dtype, self.rows(), self.N)
        if n < 0:
            from .elimination import inverse
            return inverse(self) ** (-n)
        if n == 1:
            return self
        if n % 2 == 0:
            h = self ** (n // 2)
            return h * h
        return self * (self ** (n - 1))

    def __eq__(self, other):
        return (isinstance(other, CuModArray) and self.size == other.size
                and np.array_equal(self.Array(), other.Array()))


CuModMatrix_t = CuModArray
CuModVector_t = CuModArray


def _padded_tensor(size, dtype, device="cuda"):
    if len(size) == 1:
        return torch.zeros(size[0] + TILE_WIDTH, dtype=dtype, device=device)
    return torch.zeros((size[1] + TILE_WIDTH, size[0] + TILE_WIDTH), dtype=dtype, device=device)


def CuModMatrix(A, N, mod=True, new_size=None, elem_type=DEFAULT_TYPE):
    """CuModMatrix(A, N; mod, new_size, elem_type) from a host matrix (CuModMatrix.jl:53-99,143-145):
    pads by 32 with zeros, converts to elem_type, reduces mod N on the device."""
    A = np.asarray(A)
    if A.ndim != 2:
        raise ValueError("CuModMatrix needs a 2-D array")
    if N > 2 ** 52:
        raise CuModArrayModulusMismatchException(
            "Modulus %d is bigger than 2^52 = %d, the largest supported modulus" % (N, 2 ** 52))
    data = _padded_tensor(A.shape, elem_type)
    host = torch.from_numpy(np.ascontiguousarray(A.T).astype(np.float64)).to(elem_type)
    data[: A.shape[1], : A.shape[0]].copy_(host.to(data.device, non_blocking=False))
    M = CuModArray(data, new_size or A.shape, N)
    if mod:
        mod_elements_(M)
    return M


def CuModVector(x, N, mod=True, new_size=None, elem_type=DEFAULT_TYPE):
    """CuModVector(x, N) (CuModMatrix.jl:169-171)."""
    x = np.asarray(x).reshape(-1)
    data = _padded_tensor(x.shape, elem_type)
    data[: x.shape[0]].copy_(torch.from_numpy(x.astype(np.float64)).to(elem_type).to(data.device))
    v = CuModArray(data, new_size or x.shape, N)
    if mod:
        mod_elements_(v)
    return v


def wrap(data, N, new_size=None):
    """CuModMatrix(data::CuArray, N; new_size) -- wrap existing padded device data (CuModMatrix.jl:159-161)."""
    if new_size is None:
        new_size = (data.shape[1], data.shape[0]) if data.dim() == 2 else (data.shape[0],)
    return CuModArray(data, new_size, N)


def zeros(dtype, rows, cols_or_N, N=None, new_size=None):
    """zeros(T, rows, cols, N) / zeros(T, length, N) (CuModMatrix.jl:520-534)."""
    if N is None:
        size = (rows,)
        N = cols_or_N
    else:
        size = (rows, cols_or_N)
    return CuModArray(_padded_tensor(size, dtype), new_size or size, N)


def eye(dtype, n, N):
    """eye(T, n, N) (CuModMatrix.jl:510-513)."""
    return CuModMatrix(np.eye(n, dtype=np.int64), N, elem_type=dtype)


def rand(dtype, rows, cols, N, generator=None):
    """rand(T, rows, cols, N): uniform residues (padding stays zero, unlike CuModMatrix.jl:551-556)."""
    M = zeros(dtype, rows, cols, N)
    vals = torch.randint(0, N, (cols, rows), dtype=torch.int64, device=M.data.device, generator=generator)
    M.data[:cols, :rows] = vals.to(dtype)
    return M


def similar(A, N=None):
    return CuModArray(torch.zeros_like(A.data), A.size, A.N if N is None else N)


def copy(A):
    return CuModArray(A.data.clone(), A.size, A.N)


# -- elementwise (kernel_ops/*.jl) -----------------------------------------
def _check_same(*arrs):
    s = arrs[0]
    for a in arrs[1:]:
        if a.size != s.size:
            raise CuModArraySizeMismatchException("Matrix dimensions must match")
        if a.dtype != s.dtype:
            raise TypeError("mismatched element types")


def _binary(name, C, A, B, mod_N):
    _check_same(C, A, B)
    N = mod_N if mod_N > 0 else C.N
    call("gffm_%s_%s" % (name, _sfx(C.dtype)), _ptr(C.data), _ptr(A.data), _ptr(B.data), A.padded_len, N, _stream())
    return C


def _scalar(name, C, A, s, mod_N):
    _check_same(C, A)
    N = mod_N if mod_N > 0 else C.N
    call("gffm_%s_%s" % (name, _sfx(C.dtype)), _ptr(C.data), _ptr(A.data), float(s), A.padded_len, N, _stream())
    return C


def add_(C, A, B, mod_N=-1):
    """add!(C, A, B; mod_N) (add_ops.jl:23-30)."""
    return _binary("add", C, A, B, mod_N)


def sub_(C, A, B, mod_N=-1):
    """sub!(C, A, B; mod_N) (sub_ops.jl:33-40)."""
    return _binary("sub", C, A, B, mod_N)


def elementwise_multiply_(C, A, B, mod_N=-1):
    """elementwise_multiply!(C, A, B, mod_N) (CuModMatrix.jl:564-580)."""
    if mod_N <= 0 and (A.N != B.N or A.N != C.N):
        raise CuModArrayModulusMismatchException("All matrices must have the same modulus N or provide an override mod_N")
    return _binary("mul_elementwise", C, A, B, mod_N)


def scalar_add_(C, A, s, mod_N=-1):
    return _scalar("scalar_add", C, A, s, mod_N)


def scalar_sub_(C, A, s, mod_N=-1):
    return _scalar("scalar_sub", C, A, s, mod_N)


def rscalar_sub_(C, A, s, mod_N=-1):
    return _scalar("rscalar_sub", C, A, s, mod_N)


def scalar_mul_(C, A, s, mod_N=-1):
    return _scalar("scalar_mul", C, A, s, mod_N)


def negate_(B, A, mod_N=-1):
    """negate!(B, A, mod_N) = rscalar_sub!(B, A, 0) (CuModMatrix.jl:588-605)."""
    if mod_N <= 0 and A.N != B.N:
        raise CuModArrayModulusMismatchException("Both matrices must have the same modulus N or provide an override mod_N")
    return _scalar("rscalar_sub", B, A, 0, mod_N)


def div_(C, A, s, mod_N=-1):
    """div!(C, A, s, mod_N) (kernel_ops/div_ops.jl:13-22): C = A * mod_inv(s, N) mod N."""
    N = mod_N if mod_N > 0 else C.N
    call("gffm_div_scalar_%s" % _sfx(C.dtype), _ptr(C.data), _ptr(A.data), int(s), A.padded_len, N, _stream())
    return C


def mod_(C, A, m):
    """mod!(C, A, m) (mod_ops.jl:13-21)."""
    _check_same(C, A)
    call("gffm_mod_%s" % _sfx(C.dtype), _ptr(C.data), _ptr(A.data), A.padded_len, int(m), _stream())
    return C


def mod_elements_(A, mod_N=-1):
    """mod_elements!(A, mod_N) (CuModMatrix.jl:712-716)."""
    return mod_(A, A, mod_N if mod_N > 0 else A.N)


def fill_(A, s):
    """fill!(A, s): every element (padding included, as the reference's broadcast) set to s mod N."""
    A.data.fill_(float(int(s) % A.N))
    return A


def zero_(A):
    A.data.zero_()
    return A


def copy_(B, A):
    """copy!(B, A) (CuModMatrix.jl:641-656)."""
    if A.size != B.size:
        raise CuModArraySizeMismatchException("Matrix dimensions must match")
    B.data.copy_(A.data)
    return B


def change_modulus(A, new_N):
    """change_modulus(A, new_N) (CuModMatrix.jl:730-741)."""
    R = zeros(A.dtype, *A.size, new_N) if A.ndim == 2 else zeros(A.dtype, A.size[0], new_N)
    if new_N < A.N:
        mod_(R, A, new_N)
    else:
        R.data.copy_(A.data)
    return R


def change_modulus_no_alloc_(A, new_N):
    if new_N < A.N:
        mod_(A, A, new_N)
    return CuModArray(A.data, A.size, new_N)


# -- products --------------------------------------------------------------
LIMB_MAX_N = 2 ** 26


def limbs_for(N, bits=7):
    """Digits per residue of the limb GEMM with balanced base-2^bits digits
    (csrc/k_gemm_limb.cu: limbs_for, limbs_for_bits)."""
    thresholds = (255, 65279, 16711423) if bits == 8 else (127, 16255, 2080639)
    for L, t in enumerate(thresholds, 1):
        if N <= t:
            return L
    return 4


class LimbTuning(ctypes.Structure):
    """gffm_limb_tuning: digit width (0 = the tune table's choice, 7 or 8) and grid (0 = one CTA per SM)."""
    _fields_ = [("digit_bits", ctypes.c_int32), ("max_ctas", ctypes.c_int32), ("tile_n", ctypes.c_int32),
                ("form", ctypes.c_int32)]


def _gemm(C, A, B, N, method, stripe=0, tuning=None):
    if A.dtype != B.dtype or A.dtype != C.dtype:
        raise TypeError("Mismatched element types in matmul")
    m, k = A.rows(), A.cols()
    n = B.cols()
    sfx = _sfx(C.dtype)
    if method == "auto":
        method = "limb" if 2 <= N < LIMB_MAX_N else "plain"
    if method == "limb" and tuning is not None:
        if C.dtype != torch.float64:
            raise TypeError("an explicit limb tuning takes Float64 storage")
        call("gffm_matmul_limb_tuned_f64", m, n, k, _ptr(A.data), A.ld, _ptr(B.data), B.ld, _ptr(C.data), C.ld, N,
             ctypes.byref(tuning), None, 0, _stream())
    elif method == "limb":
        call("gffm_matmul_limb_" + sfx, m, n, k, _ptr(A.data), A.ld, _ptr(B.data), B.ld, _ptr(C.data), C.ld, N,
             None, 0, _stream())
    elif method == "plain":
        call("gffm_matmul_plain_" + sfx, m, n, k, _ptr(A.data), A.ld, _ptr(B.data), B.ld, _ptr(C.data), C.ld, N,
             int(stripe or 0), _stream())
    else:
        raise ValueError("method must be 'auto', 'limb' or 'plain'")
    return C


def mul_(C, A, B, mod_N=-1, M=None, method="auto"):
    """mul!(C, A, B) (CuModMatrix.jl:767-787), mul!(z, A, x) (:816-836) and
    mul!(C, A, s, mod_N) (mul_ops.jl:170-178)."""
    if not isinstance(B, CuModArray):
        return scalar_mul_(C, A, B, mod_N)
    if A.N != B.N or A.N != C.N:
        raise CuModArrayModulusMismatchException("All matrices must have the same modulus N")
    if A.cols() != (B.rows()):
        raise CuModArraySizeMismatchException("Matrix dimensions do not match for multiplication")
    if B.ndim == 1:
        if C.size[0] != A.rows():
            raise CuModArraySizeMismatchException("Output matrix C has incorrect dimensions")
        sfx = _sfx(C.dtype)
        call("gffm_matvec_plain_" + sfx, A.rows(), A.cols(), _ptr(A.data), A.ld, _ptr(B.data), _ptr(C.data), A.N,
             int(M or 0), _stream())
        return C
    if C.rows() != A.rows() or C.cols() != B.cols():
        raise CuModArraySizeMismatchException("Output matrix C has incorrect dimensions")
    return _gemm(C, A, B, A.N, "plain" if M else method, stripe=M or 0)


def stripe_mul_(C, A, B, M=None):
    """stripe_mul!(C, A, B; M) (stripe_mul.jl:175-244): the reference's plain Float method."""
    if A.N != B.N or B.N != C.N:
        raise ValueError("Mismatched modulus in matmul")
    if A.cols() != B.rows():
        raise ValueError("DimensionMismatch")
    if B.ndim == 1:
        return mul_(C, A, B, M=M)
    return _gemm(C, A, B, A.N, "plain", stripe=M or 0)


def mat_mul_gpu_type(A, B, mod_N=-1, method="auto", tuning=None):
    """mat_mul_gpu_type(A, B, mod_N) (mat_mul_gpu_direct.jl:8-42), exact for every size.
    ``tuning``: an optional LimbTuning for the limb path."""
    N = mod_N if mod_N > 0 else A.N
    if A.cols() != B.rows():
        raise CuModArraySizeMismatchException(
            "Matrix dimensions do not match. A has %d rows and %d cols, B has %d rows and %d cols."
            % (A.rows(), A.cols(), B.rows(), B.cols()))
    C = zeros(A.dtype, A.rows(), B.cols(), N)
    return _gemm(C, A, B, N, method, tuning=tuning)


def host_matrix(A, pinned=True):
    """A host matrix (numpy array or CPU tensor of integer residues) as column-major
    Float64 storage for gffm_matmul_host_f64: a CPU tensor of shape (cols, rows),
    page-locked when ``pinned``."""
    t = torch.as_tensor(A).to(torch.float64).t().contiguous()
    return t.pin_memory() if pinned else t


def matmul_host(A, B, N, pinned=True):
    """C = A*B mod N for host matrices through gffm_matmul_host_f64 (the round trip
    CuModMatrix(A, N) * CuModMatrix(B, N) |> Array of the reference, with the copies
    overlapped with the block products).  A, B: numpy arrays or CPU tensors of
    integer values; returns an int64 numpy array."""
    A = np.asarray(A) if not torch.is_tensor(A) else A
    B = np.asarray(B) if not torch.is_tensor(B) else B
    m, k = A.shape
    k2, n = B.shape
    if k != k2:
        raise CuModArraySizeMismatchException(
            "Matrix dimensions do not match. A has %d rows and %d cols, B has %d rows and %d cols." % (m, k, k2, n))
    hA, hB = host_matrix(A, pinned), host_matrix(B, pinned)
    hC = torch.empty((n, m), dtype=torch.float64)
    if pinned:
        hC = hC.pin_memory()
    call("gffm_matmul_host_f64", m, n, k, _ptr(hA), max(m, 1), _ptr(hB), max(k, 1), _ptr(hC), max(m, 1), N,
         None, 0, _stream())
    torch.cuda.current_stream().synchronize()
    return hC.t().numpy().astype(np.int64)


def mat_mul_type_inplace_(C, A, B, mod_N=-1, method="auto"):
    """mat_mul_type_inplace!(C, A, B, mod_N) (mat_mul_gpu_direct.jl:49-85), exact, without the debug print."""
    N = mod_N if mod_N > 0 else A.N
    if C.rows() != A.rows() or C.cols() != B.cols():
        raise CuModArraySizeMismatchException("Output matrix C has incorrect dimensions")
    if A.cols() != B.rows():
        raise CuModArraySizeMismatchException("Matrix dimensions do not match.")
    return _gemm(C, A, B, N, method)


def find_max_stripe_ops(dtype, N):
    """find_max_stripe_ops(type, N) (stripe_mul.jl:13-27)."""
    bits = {torch.float64: 53, torch.float32: 24, torch.float16: 11}[dtype]
    out = ctypes.c_int64(0)
    call("gffm_find_max_stripe_ops", bits, int(N), ctypes.byref(out))
    return out.value
