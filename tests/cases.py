"""Shared seeded test inputs: (name, A, B, ncols) with numpy CSR triples.

Each case is chosen to reach particular row classes of the library (R8/R16/R32: at most
32 products per row; W: at most 128; T: at most 4096; D: more) and the edge cases the
reference's kernels have to handle: empty rows, empty B rows under non-empty A rows,
rectangular shapes, a single dense row, and products that cancel to exactly zero.
"""
import numpy as np
import scipy.sparse as sp

from opsparse_gb300 import gen


def _csr(m):
    m = sp.csr_matrix(m)
    m.sort_indices()
    m.sum_duplicates()
    return (m.indptr.astype(np.int32), m.indices.astype(np.int32), m.data.astype(np.float64))


def dense_row_case(seed=3):
    """Row 0 of A has 5000 entries pointing at B rows of ~100 entries (D class, >4096
    products), row 1 has 200 entries over short rows (T class), the rest are light."""
    rng = np.random.default_rng(seed)
    n = 20000
    A = sp.lil_matrix((50, n))
    A[0, rng.choice(n, 5000, replace=False)] = rng.standard_normal(5000)
    A[1, rng.choice(n, 200, replace=False)] = rng.standard_normal(200)
    for i in range(2, 50):
        A[i, rng.choice(n, 3, replace=False)] = rng.standard_normal(3)
    B = sp.random(n, 30000, density=100 / 30000, random_state=rng, format="csr")
    return "dense_row", _csr(A), _csr(B), 30000


def empty_b_rows_case(seed=4):
    """A rows with up to 60 entries whose B rows are mostly empty: few products but long
    A rows (not eligible for the register classes)."""
    rng = np.random.default_rng(seed)
    n = 4000
    A = sp.random(3000, n, density=0.015, random_state=rng, format="csr")
    keep = rng.random(n) < 0.05
    B = sp.random(n, 2500, density=0.004, random_state=rng, format="csr")
    B = sp.diags(keep.astype(float)) @ B
    return "empty_b_rows", _csr(A), _csr(B), 2500


def cancel_case():
    """Entries whose contributions cancel to exactly 0.0 must stay in C's pattern."""
    A = sp.csr_matrix(np.array([[1.0, 1.0, 0.0], [0.0, 2.0, -2.0], [0.0, 0.0, 0.0]]))
    B = sp.csr_matrix(np.array([[1.0, -1.0], [-1.0, 1.0], [-1.0, 1.0]]))
    return "cancel", _csr(A), _csr(B), 2


def small_cases():
    out = []
    a = gen.laplacian2d(128)
    out.append(("laplacian128", a, a, 128 * 128))
    a = gen.stencil27(12)
    out.append(("stencil27_12", a, a, 12 ** 3))
    a = gen.web_powerlaw(60000, lmax=2000)
    out.append(("web60k", a, a, 60000))
    a = gen.erdos_renyi(5000, 12.0)
    out.append(("er5k", a, a, 5000))
    a = gen.powerlaw_square(6000, 16, 2.2)
    b = gen.transpose_pattern(a[0], a[1], 6000)
    out.append(("powerlaw_AAt", a, b, 6000))
    rng = np.random.default_rng(11)
    A = sp.random(700, 300, density=0.03, random_state=rng, format="csr")
    B = sp.random(300, 900, density=0.05, random_state=rng, format="csr")
    out.append(("rect", _csr(A), _csr(B), 900))
    out.append(dense_row_case())
    out.append(empty_b_rows_case())
    out.append(cancel_case())
    return out
