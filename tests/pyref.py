"""Small pure-Python restatements used to cross-check the C oracle on tiny
inputs (a second, independent reading of the same reference functions)."""


def mod_inv(p, P):
    # src/CuModMatrix/rref_lu_pluq/pluq_kernels.jl:11-31
    inv, new_inv, rem, new_rem = 0, 1, P, p
    while new_rem != 0:
        q = rem // new_rem
        inv, new_inv = new_inv, inv - q * new_inv
        rem, new_rem = new_rem, rem - q * new_rem
    if inv < 0:
        inv += P
    return inv


def pluq(A, N):
    """pluq_gpu_kernel (src/CuModMatrix/rref_lu_pluq/pluq_kernels.jl:46-157) on a
    list-of-rows matrix; returns (U, L (m x (m+32)), row_swaps, col_swaps)."""
    m, n = len(A), len(A[0])
    A = [list(r) for r in A]
    L = [[0] * (m + 32) for _ in range(m)]
    rows_st, cols_st = [], []
    row, col, last = 0, 0, n - 1
    lsw = min(((m + 31) // 32) * 32, m + 32)
    while row < m and col < n:
        pv = pi = -1
        while True:
            colvals = [A[r][col] for r in range(row, m)]
            best = max(colvals)
            if best > 0:
                pv, pi = best, row + colvals.index(best)
                break
            for r in range(m):
                A[r][col], A[r][last] = A[r][last], A[r][col]
            cols_st.append((col + 1, last + 1))
            col += 1
            if col >= n:
                break
        if col >= n:
            break
        inv = mod_inv(pv, N)
        old_p = A[pi][:n]
        A[pi][:n] = A[row][:n]
        A[row][:n] = [(x * inv) % N for x in old_p]
        if pi != row:
            L[row][:lsw], L[pi][:lsw] = L[pi][:lsw], L[row][:lsw]
            rows_st.append((row + 1, pi + 1))
        L[row][col] = pv
        for r in range(row + 1, m):
            L[r][col] = A[r][col]
            A[r][col] = 0
        for r in range(row + 1, m):
            mlt = N - L[r][col]
            for c in range(col + 1, n):
                A[r][c] = (A[r][c] + mlt * A[row][c]) % N
        row += 1
        col += 1
    return A, L, rows_st, cols_st


def matmul(A, B, N):
    return [[sum(A[i][p] * B[p][j] for p in range(len(B))) % N for j in range(len(B[0]))] for i in range(len(A))]


def inverse_mod(A, N):
    """Gauss-Jordan inverse mod prime N (None when singular)."""
    n = len(A)
    M = [list(r) + [int(i == j) for j in range(n)] for i, r in enumerate(A)]
    for c in range(n):
        pr = next((r for r in range(c, n) if M[r][c] % N), None)
        if pr is None:
            return None
        M[c], M[pr] = M[pr], M[c]
        iv = pow(M[c][c], -1, N)
        M[c] = [(x * iv) % N for x in M[c]]
        for r in range(n):
            if r != c and M[r][c]:
                f = M[r][c]
                M[r] = [(x - f * y) % N for x, y in zip(M[r], M[c])]
    return [r[n:] for r in M]


# ---- Karatsuba kernels as the reference writes them (Julia rem / mod / div) ----
def _rem(a, b):
    """Julia rem / %: the sign of the dividend."""
    r = abs(a) % abs(b)
    return r if a >= 0 else -r


def _div(a, b):
    """Julia div: truncating division."""
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b >= 0) else -q


def kara_add(a1, a2, b1, b2, N1, N2):
    # karatsuba_add_helper (src/KaratsubaMatrix/KaratsubaKernels.jl:2-17)
    temp = _rem(a1 + b1, 2 * N1)
    temp = _div(temp, N1)
    res2 = _rem(temp + a2, 2 * N2)
    res2 = _rem(res2 + b2, 2 * N2)
    temp = _rem(temp * N1, N1 ** 2)
    temp = _rem(b1 - temp, N1 ** 2)
    res1 = _rem(a1 + temp, N1 ** 2)
    return _rem(res1, N1), _rem(res2, N2)


def kara_negate(a1, a2, N1, N2, M):
    # karatsuba_negate_helper (KaratsubaKernels.jl:79-97)
    res2 = _rem(0, N2)
    res2 = _rem(res2 + N1, 2 * N1)
    res2 = _rem(res2 - a1, 2 * N1)
    res2 = _div(res2, N1)
    res1 = _rem(res2 * N1, M ** 2)
    res1 = _rem(res1 + a1, M ** 2)
    res1 = _rem(-res1, N1)
    res1 = res1 % N1
    res2 = _rem(res2 + N2, M ** 2)
    res2 = _rem(res2 - 1, M ** 2)
    res2 = _rem(res2 - a2, M)
    return res1, _rem(res2, N2)


def kara_sub(a1, a2, b1, b2, N1, N2, M):
    # karatsuba_sub_kernel! (KaratsubaKernels.jl:113-125): negate B, then add A
    n1, n2 = kara_negate(b1, b2, N1, N2, M)
    return kara_add(n1, n2, a1, a2, N1, N2)


def kara_scalar(a1, a2, s, N1, N2):
    # karatsuba_scalar_multiply_helper (KaratsubaKernels.jl:52-60)
    res2 = _rem(a1 * s, N1 ** 2)
    res2 = _div(res2, N1)
    res1 = _rem(a2 * s, N2)
    res2 = _rem(res2 + res1, N2)
    res1 = _rem(a1 * s, N1)
    return res1, res2


def kara_matmul(A1, A2, B1, B2, N1, N2):
    """KMatMul! (src/KaratsubaMatrix/KaratsubaMatrix.jl:133-204) with its kernels
    karatsuba_matmul_kernel_1!/2! (KaratsubaKernels.jl:129-158), products exact
    (the reference's striped Float64 mul! is exact for these bounds)."""
    m, k, n = len(A1), len(A1[0]), len(B1[0])
    Ap = [[_rem(A1[i][p] + A2[i][p], 2 * N1) for p in range(k)] for i in range(m)]
    Bp = [[_rem(B1[p][j] + B2[p][j], 2 * N1) for j in range(n)] for p in range(k)]

    def mm(X, Y, P):
        return [[sum(X[i][p] * Y[p][j] for p in range(k)) % P for j in range(n)] for i in range(m)]

    C1 = mm(A1, B1, N1 ** 2)                 # mul!(C.data1, A.data1, B.data1, R=N1, P=N1^2)
    C2 = mm(Ap, Bp, (4 * N1) ** 2)           # mul!(C.data2, A.plan, B.plan, R=2N1, P=(4N1)^2)
    T = mm(A2, B2, N1 ** 2)                  # mul!(B.plan, A.data2, B.data2, R=N1, P=N1^2)
    R1 = [[0] * n for _ in range(m)]
    R2 = [[0] * n for _ in range(m)]
    Q = (4 * N1) ** 2
    for i in range(m):
        for j in range(n):
            cc1 = C1[i][j] % (N1 ** 2)
            cc2 = C2[i][j] % Q
            bp = T[i][j] % N1
            cp = _div(cc1, N1)
            cc2 = _rem(cc2 - cc1, Q)
            cc2 = _rem(cc2 - bp, Q)
            cc2 = cc2 + cp
            R1[i][j] = cc1 % N1
            R2[i][j] = cc2 % N2
    return R1, R2


def tri_window(A, N, rs, cs, upper):
    """forward_sub_kernel_32 / backward_sub_kernel_32 (src/CuModMatrix/triangular/
    substitution_inplace.jl:6-35, 63-88) on a list-of-rows matrix, entries outside
    A read as the zero padding; returns the 32 x 32 window result."""
    m, n = len(A), (len(A[0]) if A else 0)

    def at(i, j):
        return A[i][j] % N if 0 <= i < m and 0 <= j < n else 0

    X = [[0] * 32 for _ in range(32)]
    for c in range(32):
        rows = range(31, -1, -1) if upper else range(32)
        for r in rows:
            ks = range(r + 1, 32) if upper else range(r)
            s = sum(at(rs + r, cs + k) * X[k][c] for k in ks) % N
            rhs = 1 if r == c else 0
            X[r][c] = mod_inv(at(rs + r, rs + r), N) * (rhs - s + N) % N
    return X


def tri_inverse(A, N, upper):
    """upper/lower_triangular_inverse_no_copy (triangular_inverse_no_copy.jl:18-477),
    following the reference's three branches literally; returns the (n x m) result
    as a list of rows, or None for the InverseNotDefinedException case."""
    m, n = len(A), len(A[0])
    X = [[0] * m for _ in range(n)]
    if (m <= 32) if upper else (n <= 32):
        W = tri_window(A, N, 0, 0, upper)
        for r in range(min(32, n)):
            for c in range(min(32, m)):
                X[r][c] = W[r][c]
        return X
    if not upper and m > n:
        return None

    def put_window(lo, size):
        W = tri_window(A, N, lo, lo, upper)
        for r in range(size):
            for c in range(size):
                X[lo + r][lo + c] = W[r][c]

    def combine(lo, mid, hi):
        if upper:      # X12 = -(X11 A12) X22
            T = [[sum(X[i][t] * A[t][j] for t in range(lo, mid)) % N for j in range(mid, hi)] for i in range(lo, mid)]
            for i in range(lo, mid):
                for j in range(mid, hi):
                    X[i][j] = (N - sum(T[i - lo][t - mid] * X[t][j] for t in range(mid, hi)) % N) % N
        else:          # X21 = -(X22 A21) X11
            T = [[sum(X[i][t] * A[t][j] for t in range(mid, hi)) % N for j in range(lo, mid)] for i in range(mid, hi)]
            for i in range(mid, hi):
                for j in range(lo, mid):
                    X[i][j] = (N - sum(T[i - mid][t - lo] * X[t][j] for t in range(lo, mid)) % N) % N

    def rec(lo, hi):
        if hi - lo <= 32:                                  # first branch
            put_window(lo, hi - lo)
            return
        q = max(int((hi - lo) / 64 + 0.5), 1)
        mid = lo + 32 * q
        if mid - lo <= 32 and hi - mid <= 32:              # second branch: both halves by window
            put_window(lo, mid - lo)
            put_window(mid, hi - mid)
        else:                                              # third branch
            rec(lo, mid)
            rec(mid, hi)
        combine(lo, mid, hi)

    rec(0, min(m, n))
    return X
