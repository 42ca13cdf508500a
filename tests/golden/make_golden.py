"""Generate tests/golden/reference_kat.json -- the known-answer vectors of the
reference's own test-suite, transcribed with their source lines.

The reference (GPUFiniteFieldMatrices.jl) is Julia and cannot run in this
environment, so every expected value here is computed the way the reference
test itself states it (e.g. ``mod.(A_data * B_data, modulus)``), with exact
Python integers.  Matrices are written row by row (the way they read in the
Julia source).  Run:  python tests/golden/make_golden.py
"""
import json
import os


def mat_mul(A, B):
    return [[sum(A[i][p] * B[p][j] for p in range(len(B))) for j in range(len(B[0]))] for i in range(len(A))]


def mod(A, N):
    return [[x % N for x in row] for row in A]


def elementwise(A, B, f):
    return [[f(a, b) for a, b in zip(ra, rb)] for ra, rb in zip(A, B)]


def main():
    kat = {"source": "GPUFiniteFieldMatrices.jl test suite (paths inside that repository)", "cases": []}
    add = kat["cases"].append

    # test/CuModMatrix/matmul_operations_test.jl:14-17 (A*B mod 11) and :54-67 (override mod 7)
    A = [[1, 2, 3], [4, 5, 6]]
    B = [[7, 8], [9, 10], [0, 1]]
    add({"op": "matmul", "src": "test/CuModMatrix/matmul_operations_test.jl:14-17,40-42",
         "A": A, "B": B, "N": 11, "expected": mod(mat_mul(A, B), 11)})
    add({"op": "matmul_override", "src": "test/CuModMatrix/matmul_operations_test.jl:54-67",
         "A": A, "B": B, "N_storage": 11, "N": 7, "expected": mod(mat_mul(A, B), 7)})
    # :79-126 in-place product mod 9 (B holds 11, 12 >= 9: reduced on construction) and override mod 3
    B2 = [[7, 8], [9, 10], [11, 12]]
    add({"op": "matmul", "src": "test/CuModMatrix/matmul_operations_test.jl:79-108",
         "A": A, "B": B2, "N": 9, "expected": mod(mat_mul(A, B2), 9)})
    add({"op": "matmul_override", "src": "test/CuModMatrix/matmul_operations_test.jl:110-122",
         "A": A, "B": B2, "N_storage": 9, "N": 3, "expected": mod(mat_mul(A, B2), 3)})

    # test/CuModMatrix/basic_operations_test.jl:18-118 and inplace_operations_test.jl:16-107
    A = [[1, 2, 3], [4, 5, 6], [7, 8, 9]]
    B = [[9, 8, 7], [6, 5, 4], [3, 2, 1]]
    N = 11
    src_b = "test/CuModMatrix/basic_operations_test.jl"
    src_i = "test/CuModMatrix/inplace_operations_test.jl"
    add({"op": "add", "src": src_b + ":48-55; " + src_i + ":32-38", "A": A, "B": B, "N": N,
         "expected": mod(elementwise(A, B, lambda a, b: a + b), N)})
    add({"op": "sub", "src": src_b + ":57-66; " + src_i + ":40-46", "A": A, "B": B, "N": N,
         "expected": mod(elementwise(A, B, lambda a, b: a - b), N)})
    add({"op": "matmul", "src": src_b + ":68-77", "A": A, "B": B, "N": N, "expected": mod(mat_mul(A, B), N)})
    add({"op": "elementwise_mul", "src": src_b + ":79-89; " + src_i + ":48-54", "A": A, "B": B, "N": N,
         "expected": mod(elementwise(A, B, lambda a, b: a * b), N)})
    add({"op": "scalar_add", "src": src_b + ":94-101; " + src_i + ":67-73", "A": A, "s": 3, "N": N,
         "expected": mod([[a + 3 for a in r] for r in A], N)})
    add({"op": "scalar_sub", "src": src_b + ":103-110; " + src_i + ":75-80", "A": A, "s": 3, "N": N,
         "expected": mod([[a - 3 for a in r] for r in A], N)})
    add({"op": "scalar_mul", "src": src_b + ":112-119; " + src_i + ":82-88", "A": A, "s": 3, "N": N,
         "expected": mod([[a * 3 for a in r] for r in A], N)})
    add({"op": "scalar_mul", "src": src_b + ":121-128 (A * -1)", "A": A, "s": -1, "N": N,
         "expected": mod([[-a for a in r] for r in A], N)})
    add({"op": "negate", "src": src_i + ":56-62", "A": A, "N": N,
         "expected": mod([[-a for a in r] for r in A], N)})
    # modulus override, inplace_operations_test.jl:125-193
    A = [[1, 5, 10], [15, 20, 25], [30, 35, 40]]
    add({"op": "add", "src": src_i + ":125-143 (storage mods 27 and 9, override 3)", "A": mod(A, 27),
         "B": mod(A, 9), "N": 3, "expected": mod(elementwise(A, A, lambda a, b: a + b), 3)})
    add({"op": "sub", "src": src_i + ":145-152", "A": mod(A, 27), "B": mod(A, 9), "N": 3,
         "expected": mod(elementwise(A, A, lambda a, b: a - b), 3)})
    add({"op": "elementwise_mul", "src": src_i + ":154-161", "A": mod(A, 27), "B": mod(A, 9), "N": 3,
         "expected": mod(elementwise(A, A, lambda a, b: a * b), 3)})
    add({"op": "scalar_add", "src": src_i + ":165-172", "A": mod(A, 27), "s": 3, "N": 3,
         "expected": mod([[a + 3 for a in r] for r in A], 3)})
    add({"op": "scalar_sub", "src": src_i + ":174-181", "A": mod(A, 27), "s": 3, "N": 3,
         "expected": mod([[a - 3 for a in r] for r in A], 3)})
    add({"op": "scalar_mul", "src": src_i + ":183-190", "A": mod(A, 27), "s": 3, "N": 3,
         "expected": mod([[a * 3 for a in r] for r in A], 3)})
    # mod_elements!, inplace_operations_test.jl:225-245; fill!, :247-251
    A = [[1, 2, 3], [4, 5, 6], [7, 8, 9]]
    A2 = [[2 * a for a in r] for r in A]
    add({"op": "mod", "src": src_i + ":225-236 (CuModMatrix(A*2, 11) then mod_elements!)", "A": A2, "N": 11,
         "expected": mod(A2, 11)})
    add({"op": "mod", "src": src_i + ":238-245 (override 5)", "A": mod(A2, 11), "N": 5,
         "expected": mod(mod(A2, 11), 5)})
    add({"op": "fill", "src": src_i + ":247-251", "shape": [3, 3], "s": 122, "N": 11,
         "expected": [[122 % 11] * 3 for _ in range(3)]})
    # change_modulus, basic_operations_test.jl:221-260
    add({"op": "mod", "src": src_b + ":221-260 (change_modulus to 7)", "A": A, "N": 7, "expected": mod(A, 7)})
    # matrix power, basic_operations_test.jl:161-199
    G = [[1, 2, 3], [0, 1, 4], [5, 6, 0]]
    add({"op": "matmul", "src": src_b + ":161-193 (G^2)", "A": G, "B": G, "N": 11,
         "expected": mod(mat_mul(G, G), 11)})

    # test/CuModMatrix/permutation_test.jl:3-55
    P3 = [[1, 2, 3], [4, 5, 6], [7, 8, 9]]
    add({"op": "col_perm", "src": "test/CuModMatrix/permutation_test.jl:3-23", "A": P3, "swaps": [[2, 3]],
         "N": 11, "expected": [[1, 3, 2], [4, 6, 5], [7, 9, 8]]})
    add({"op": "row_perm", "src": "test/CuModMatrix/permutation_test.jl:33-45", "A": P3, "swaps": [[2, 3]],
         "N": 11, "expected": [[1, 2, 3], [7, 8, 9], [4, 5, 6]]})

    # test/CuModMatrix/de_rham_test.jl:3-37: invertible mod 7, A * A^-1 = I
    D = [[0, 0, 0, 0, 0, 0, 0, -3, 0, 0],
         [0, 0, 0, 0, 0, 0, 0, 0, -3, 0],
         [0, 1, 0, 0, 0, 0, 0, 0, 0, 0],
         [0, 0, 1, 0, 0, 0, 0, 0, 0, 0],
         [0, -2, 0, 0, 0, 0, 0, 0, 0, -3],
         [0, 0, -2, 0, 2, 0, 0, 0, 0, 0],
         [0, 0, 0, 1, 0, 2, 0, 0, 0, 0],
         [0, -3, 0, -2, 0, 0, 0, -1, 0, 0],
         [0, 0, -3, 0, 0, 0, 2, 0, -1, 0],
         [1, 0, 0, -3, 0, 0, 0, 0, 0, -1]]
    add({"op": "invertible", "src": "test/CuModMatrix/de_rham_test.jl:3-37", "A": mod(D, 7), "N": 7,
         "expected_invertible": True,
         "expected_product_with_inverse": [[int(i == j) for j in range(10)] for i in range(10)]})
    # test/CuModMatrix/subst_test.jl:5-116: 6x6 identity mod 11, P^-1 L U Q^-1 = A, A^-1 A = I
    I6 = [[int(i == j) for j in range(6)] for i in range(6)]
    add({"op": "invertible", "src": "test/CuModMatrix/subst_test.jl:5-116", "A": I6, "N": 11,
         "expected_invertible": True, "expected_product_with_inverse": I6})
    # basic_operations_test.jl:204 (commented check): linearly dependent rows are not invertible
    add({"op": "invertible", "src": src_b + ":203-214", "A": [[1, 2, 3], [2, 4, 6], [3, 6, 9]], "N": 11,
         "expected_invertible": False})

    # test/KaratsubaMatrix/basic_operations_test.jl:51-65: digits base 100 of Z/100^2
    A = [[1, 2], [3, 4]]
    B = [[5, 6], [7, 8]]
    add({"op": "karatsuba_matmul", "src": "test/KaratsubaMatrix/basic_operations_test.jl:51-65 (A*B)",
         "A1": A, "A2": [[0, 0], [0, 0]], "B1": B, "B2": [[0, 0], [0, 0]], "N1": 100, "N2": 100,
         "expected_value": mod(mat_mul(A, B), 100 * 100)})
    add({"op": "karatsuba_add", "src": "test/KaratsubaMatrix/basic_operations_test.jl:51-65 (A+B)",
         "A1": A, "A2": [[0, 0], [0, 0]], "B1": B, "B2": [[0, 0], [0, 0]], "N1": 100, "N2": 100,
         "expected_value": mod(elementwise(A, B, lambda a, b: a + b), 100 * 100)})
    add({"op": "karatsuba_sub", "src": "test/KaratsubaMatrix/basic_operations_test.jl:51-65 (A-B)",
         "A1": A, "A2": [[0, 0], [0, 0]], "B1": B, "B2": [[0, 0], [0, 0]], "N1": 100, "N2": 100,
         "expected_value": mod(elementwise(A, B, lambda a, b: a - b), 100 * 100)})
    add({"op": "karatsuba_scalar", "src": "test/KaratsubaMatrix/basic_operations_test.jl:51-64 (a*A, a = 9)",
         "A1": A, "A2": [[0, 0], [0, 0]], "s": 9, "N1": 100, "N2": 100,
         "expected_value": mod([[9 * x for x in row] for row in A], 100 * 100)})
    C1 = [[1, 0, 3], [8, 11, 2], [2, 4, 6]]
    C2 = [[10, 3, 2], [7, 13, 7], [1, 0, 9]]
    D1 = [[9, 6, 5], [2, 17, 9], [4, 4, 23]]
    D2 = [[5, 5, 11], [6, 4, 3], [7, 3, 19]]
    vC = [[a + 100 * b for a, b in zip(r1, r2)] for r1, r2 in zip(C1, C2)]
    vD = [[a + 100 * b for a, b in zip(r1, r2)] for r1, r2 in zip(D1, D2)]
    src_k = "test/KaratsubaMatrix/basic_operations_test.jl:56-70 (CK, DK digit matrices)"
    add({"op": "karatsuba_matmul", "src": src_k, "A1": C1, "A2": C2, "B1": D1, "B2": D2, "N1": 100, "N2": 100,
         "expected_value": mod(mat_mul(vC, vD), 100 * 100)})
    add({"op": "karatsuba_add", "src": src_k, "A1": C1, "A2": C2, "B1": D1, "B2": D2, "N1": 100, "N2": 100,
         "expected_value": mod(elementwise(vC, vD, lambda a, b: a + b), 100 * 100)})
    add({"op": "karatsuba_sub", "src": src_k, "A1": C1, "A2": C2, "B1": D1, "B2": D2, "N1": 100, "N2": 100,
         "expected_value": mod(elementwise(vC, vD, lambda a, b: a - b), 100 * 100)})

    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kat.json")
    with open(out, "w") as f:
        json.dump(kat, f, indent=1)
    print("wrote", out, len(kat["cases"]), "cases")


if __name__ == "__main__":
    main()
