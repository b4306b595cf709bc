"""Parity at the benchmark configurations' full sizes: every result the benchmarks time is
checked against the oracle on the same inputs, and its measured error is reported (a
"PARITY {...}" line per result at the end of the pytest run).

  C1  2-D Laplacian 128 x 128, FP64: bit-exact structure and values.
  C2  1,000,000-row web-like power-law graph, FP64: bit-exact (ops_spgemm, one pass).
  C3  27-point stencil 80^3 (512,000 rows, 61,162,984 outputs of up to 125 entries), FP64
      bit-exact; FP32 bit-identical to the oracle's FP32 (Dot2) and within 1e-5 of the FP64
      oracle (relative to each entry, or to 2^-24 * sum|a*b| of its terms where they cancel).
  C5  forward of A * B, A 200,000^2 power law (mean degree 16, exponent 2.2), B = pattern
      of A^T with fresh values: FP64 bit-exact, FP32 as C3; plus the backward's dA, dB.
  C4  4,096 Erdos-Renyi problems (sizes log-uniform in 64..65,536, mean degree U(4,32)),
      FP32, one batch: every problem's result equals the single call's bit for bit (on the
      device), and a seeded sample of 48 problems matches the oracle as C3's FP32.
Tolerances: FP64 1e-12 relative, FP32 1e-5 relative.
"""
import numpy as np
import pytest

import bench
import oracle
import opsparse_gb300 as ops
from opsparse_gb300 import gen
from tests.parity_log import RECORDS as PARITY_RECORDS

pytestmark = pytest.mark.gpu


def _record(name, rep):
    rec = dict(config=name, **{k: v for k, v in rep.items() if k != "checked_against"})
    PARITY_RECORDS.append(rec)
    return rec


def _check(name, rep, dt, bit_exact_f32=None):
    rec = _record(name, rep)
    assert rep["structure_identical"], rec
    assert rep["within_tolerance"], rec
    if dt == "f64":
        assert rep["values_bit_identical"], rec
    if bit_exact_f32 is not None:
        assert bit_exact_f32, rec


def _run(cuda, a, b, ncols, dtype, one_pass=1):
    A = ops.csr_to_device(*a, len(a[0]) - 1, len(b[0]) - 1, dtype=dtype)
    B = A if b is a else ops.csr_to_device(*b, len(b[0]) - 1, ncols, dtype=dtype)
    with ops.Handle() as h:
        h.set_one_pass(one_pass)
        C = h.spgemm_oneshot(A, B)
        res = C.to_host()
    del A, B, C
    cuda.cuda.empty_cache()
    return res


def _abs_sums(a, b):
    """sum_j |a_ij b_jk| per output entry (the OpenMP port over |A|, |B|: same structure)."""
    return lambda: oracle.omp_spgemm(a[0], a[1], np.abs(a[2].astype(np.float64)), b[0], b[1],
                                     np.abs(b[2].astype(np.float64)))[2]


def _f64_and_f32(cuda, name, a, b, ncols):
    gpu = _run(cuda, a, b, ncols, cuda.float64)
    ref = oracle.spgemm(*a, *b, ncols)
    _check(f"{name}/f64", bench.parity_report(gpu, ref, "f64"), "f64")
    a32 = (a[0], a[1], a[2].astype(np.float32))
    b32 = a32 if b is a else (b[0], b[1], b[2].astype(np.float32))
    gpu32 = _run(cuda, a32, a32 if b is a else b32, ncols, cuda.float32)
    ref32 = oracle.spgemm(*a32, *b32, ncols, dtype=np.float32)
    ref64 = oracle.spgemm(a[0], a[1], a32[2].astype(np.float64), b[0], b[1], b32[2].astype(np.float64), ncols)
    dot2_identical = bool(np.array_equal(gpu32[2].view(np.uint32), ref32[2].view(np.uint32)))
    rep = bench.parity_report(gpu32, ref64, "f32", scale_fn=_abs_sums(a32, b32))
    rep["values_bit_identical_to_fp32_oracle"] = dot2_identical
    _check(f"{name}/f32", rep, "f32", bit_exact_f32=dot2_identical)


def test_c1_laplacian_128(cuda):
    a = gen.laplacian2d(128)
    n = len(a[0]) - 1
    gpu = _run(cuda, a, a, n, cuda.float64)
    ref = oracle.spgemm(*a, *a, n)
    assert len(ref[1]) == 210_436
    _check("C1 laplacian2d_128", bench.parity_report(gpu, ref, "f64"), "f64")


def test_c2_web_powerlaw_1m(cuda):
    a = gen.web_powerlaw()
    n = len(a[0]) - 1
    for one_pass in (1, 0):
        gpu = _run(cuda, a, a, n, cuda.float64, one_pass=one_pass)
        ref = oracle.spgemm(*a, *a, n)
        _check(f"C2 web_powerlaw_1M/{'one' if one_pass else 'two'}_pass", bench.parity_report(gpu, ref, "f64"),
               "f64")


def test_c3_stencil27_80(cuda):
    a = gen.stencil27(80)
    n = len(a[0]) - 1
    assert len(a[1]) == 13_481_272
    _f64_and_f32(cuda, "C3 stencil27_80^3", a, a, n)


def test_c5_powerlaw_aat_forward_and_backward(cuda):
    torch = cuda
    n = 200_000
    a = gen.powerlaw_square(n, 16, 2.2)
    b = gen.transpose_pattern(a[0], a[1], n)
    _f64_and_f32(cuda, "C5 powerlaw_200k_AAt forward", a, b, n)
    # the backward of the same product: dA, dB bit-identical to the oracle's
    from opsparse_gb300.autograd import FixedPatternSpGEMM

    A = ops.csr_to_device(*a, n, n, dtype=torch.float64)
    B = ops.csr_to_device(*b, n, n, dtype=torch.float64)
    with ops.Handle() as h:
        op = FixedPatternSpGEMM(A, B, h)
        op.forward_values(A.val, B.val)
        w = torch.as_tensor(np.random.default_rng(3).standard_normal(op.nnz)).cuda()
        da, db = op.backward_values(A.val, B.val, w)
        crpt, ccol = op.c_rpt.cpu().numpy(), op.c_col.cpu().numpy()
        da, db, w = da.cpu().numpy(), db.cpu().numpy(), w.cpu().numpy()
    oda, odb = oracle.backward(*a, *b, n, crpt.astype(np.int64), ccol, w)
    for nm, g, o in (("dA", da, oda), ("dB", db, odb)):
        diff = np.abs(g - o)
        nz = o != 0
        rec = _record(f"C5 powerlaw_200k_AAt backward {nm}/f64",
                      {"structure_identical": True, "entries": int(o.size), "max_abs_err": float(diff.max()),
                       "max_rel_err": float((diff[nz] / np.abs(o[nz])).max()) if nz.any() else 0.0,
                       "values_bit_identical": bool(np.array_equal(g.view(np.uint64), o.view(np.uint64)))})
        assert rec["values_bit_identical"], rec


def test_c4_batched_4096(cuda):
    torch = cuda
    from opsparse_gb300 import gen_device

    sizes, row_base, a_side, b_side = gen_device.er_batch(4096, dtype=torch.float32)
    A = gen_device.problem_slices(sizes, row_base, a_side)
    B = gen_device.problem_slices(sizes, row_base, b_side)
    pairs = [(ops.CsrMatrix(int(n), int(n), ar, ac, av), ops.CsrMatrix(int(n), int(n), br, bc, bv))
             for (ar, ac, av, _), (br, bc, bv, _), n in zip(A, B, sizes)]
    h = ops.Handle()
    batch = ops.Batch(h, pairs)
    batch.execute(True)
    batch.check()
    single = ops.Handle()
    mism = []
    for i, (Ap, Bp) in enumerate(pairs):
        c = single.spgemm_oneshot(Ap, Bp)
        rpt, col, val, nnz = batch.result_device(i)
        if not (nnz == c.nnz and torch.equal(rpt, c.rpt) and torch.equal(col, c.col)
                and torch.equal(val.view(torch.int32), c.val.view(torch.int32))):
            mism.append(i)
        del c
    seg, flop, nnz_total = batch.info()
    _record("C4 batched_er_4096 vs per-call results", {"problems": len(pairs), "products": flop, "nnz": nnz_total,
                                                       "problems_differing": len(mism)})
    assert not mism, mism[:10]
    sample = np.random.default_rng(20261203).choice(len(pairs), 48, replace=False)
    worst = {"structure_identical": True, "within_tolerance": True, "max_abs_err": 0.0, "max_rel_err_scaled": 0.0,
             "entries": 0, "values_bit_identical_to_fp32_oracle": True}
    for i in sample:
        Ap, Bp = pairs[i]
        a = tuple(x.cpu().numpy() for x in (Ap.rpt, Ap.col, Ap.val))
        b = tuple(x.cpu().numpy() for x in (Bp.rpt, Bp.col, Bp.val))
        gpu = batch.result(int(i))
        ref32 = oracle.spgemm(*a, *b, Bp.cols, dtype=np.float32)
        ref64 = oracle.spgemm(a[0], a[1], a[2].astype(np.float64), b[0], b[1], b[2].astype(np.float64), Bp.cols)
        rep = bench.parity_report(gpu, ref64, "f32", scale_fn=_abs_sums(a, b))
        worst["structure_identical"] &= rep["structure_identical"]
        worst["within_tolerance"] &= bool(rep.get("within_tolerance", False))
        worst["max_abs_err"] = max(worst["max_abs_err"], rep.get("max_abs_err", np.inf))
        worst["max_rel_err_scaled"] = max(worst["max_rel_err_scaled"], rep.get("max_rel_err_scaled") or 0.0)
        worst["entries"] += rep.get("entries", 0)
        worst["values_bit_identical_to_fp32_oracle"] &= bool(
            np.array_equal(gpu[2].view(np.uint32), ref32[2].view(np.uint32)))
    rec = _record("C4 batched_er_4096 sample of 48 vs oracle/f32", worst)
    batch.close()
    assert worst["structure_identical"] and worst["within_tolerance"], rec
    assert worst["values_bit_identical_to_fp32_oracle"], rec
