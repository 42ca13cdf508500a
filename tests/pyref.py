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
