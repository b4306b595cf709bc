"""Generates tests/golden/*.npz: small seeded inputs together with the outputs of
OpSparse's own SpGEMM kernels (compiled from its sources and run on the CPU by
oracle/ref_emul) and of its host compute_flop.

Run where the OpSparse source tree is (OPSPARSE_SRC=<dir>, or the default of
oracle/ref_emul/Makefile):
    python tests/golden/make_golden.py
Each fixture holds a_rpt/a_col/a_val, b_rpt/b_col/b_val, ncols, the reference's
c_rpt/c_col/c_val, its per-row flop counts, and the bin histograms its binning kernels
produced (symbolic and numeric) plus how many rows took its global-hash fallback.
"""
import sys
from pathlib import Path

import numpy as np
import scipy.sparse as sp

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from opsparse_gb300 import gen  # noqa: E402
from oracle import ref  # noqa: E402

OUT = Path(__file__).resolve().parent


def _csr(m):
    m = sp.csr_matrix(m)
    m.sum_duplicates()
    m.sort_indices()
    return m.indptr.astype(np.int32), m.indices.astype(np.int32), m.data.astype(np.float64)


def cases():
    out = {}
    a = gen.laplacian2d(32)
    out["laplacian32"] = (a, a, 32 * 32)
    a = gen.stencil27(7)
    out["stencil27_7"] = (a, a, 7 ** 3)
    a = gen.web_powerlaw(3000, lmax=400, window=64)
    out["web3k"] = (a, a, 3000)
    a = gen.erdos_renyi(600, 8.0)
    out["er600"] = (a, a, 600)
    p = gen.powerlaw_square(1000, 8, 2.2)
    out["powerlaw_AAt"] = (p, gen.transpose_pattern(p[0], p[1], 1000), 1000)
    rng = np.random.default_rng(5)
    A = sp.random(300, 120, density=0.04, random_state=rng, format="csr")
    B = sp.random(120, 410, density=0.05, random_state=rng, format="csr")
    out["rect"] = (_csr(A), _csr(B), 410)
    # a ladder of heavy rows (x12 products each): row 0 has ~30,000 products over 60,000
    # columns, more distinct columns than 0.8 of the reference's largest shared table
    # (19,660) -> its global-hash fallback (symbolic) and global numeric table; rows 1-4
    # land in its symbolic bins 3-6 and numeric bins 5-7
    n = 6000
    A = sp.lil_matrix((14, n))
    for i, k in enumerate((2500, 120, 200, 400, 700)):
        A[i, rng.choice(n, k, replace=False)] = rng.standard_normal(k)
    for i in range(5, 14):
        A[i, rng.choice(n, 4, replace=False)] = rng.standard_normal(4)
    B = sp.random(n, 60000, density=12 / 60000, random_state=rng, format="csr")
    out["dense_row"] = (_csr(A), _csr(B), 60000)
    A = np.array([[1.0, 1.0, 0.0], [0.0, 2.0, -2.0], [0.0, 0.0, 0.0]])
    B = np.array([[1.0, -1.0], [-1.0, 1.0], [-1.0, 1.0]])
    out["cancel"] = (_csr(A), _csr(B), 2)
    return out


def main():
    for name, (a, b, ncols) in cases().items():
        crpt, ccol, cval, info = ref.spgemm(*a, *b, ncols)
        tot, rf = ref.compute_flop(a[0], a[1], b[0])
        np.savez_compressed(OUT / f"{name}.npz", a_rpt=a[0], a_col=a[1], a_val=a[2], b_rpt=b[0], b_col=b[1],
                            b_val=b[2], ncols=np.int64(ncols), c_rpt=crpt, c_col=ccol, c_val=cval, row_flop=rf,
                            total_flop=np.int64(tot), bins_symbolic=np.array(info["bins_symbolic"]),
                            bins_numeric=np.array(info["bins_numeric"]),
                            global_fallback_rows=np.int64(info["global_fallback_rows"]))
        print(f"{name}: nnz(C)={len(ccol)} flop={tot} {info}")


if __name__ == "__main__":
    main()
