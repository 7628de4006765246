"""Radiance storage precision at its own full-size workload, against the FP64 oracle.

64x64x32 blocks, every probe (131,072) each pass, 256 rays, max_dist 256, blend 0.1, 16 passes
from a zero volume; FP32, FP16 and BF16 storage with FP32 arithmetic.  The FP64 oracle keeps the
traversal in FP32/int (hit records must be bit-exact at every storage precision, checked on a 2%
probe subset) and does shading, trilinear taps, reduction and blend in double.  Error of a
channel: |gpu - oracle| / max(|oracle|, 1e-3).  Each pass reads the previous pass's rounded
volume (shaders/radiance.comp:349-354 stores every pass), so the 16-bit errors compound; the
bounds below are the per-pass rounding (2^-11 for FP16, 2^-8 for BF16) compounded over 16 passes
with margin.
"""
import pytest

pytestmark = pytest.mark.gpu

# (max rel of pass 1, max rel worst of 16 passes, RMS rel worst of 16 passes)
BOUNDS = {"fp32": (1e-5, 1e-5, 1e-6), "fp16": (1e-3, 2e-3, 5e-4), "bf16": (5e-3, 1.6e-2, 4e-3)}


def test_storage_precision_full_size_vs_fp64():
    from tests import precision_report
    m = precision_report.measure()
    assert m["probes"] == 64 * 64 * 32
    for prec, ok in m["hits_ok"].items():
        assert ok, f"{prec}: hit records differ from the FP64 oracle"
    for prec, (b1, bmax, brms) in BOUNDS.items():
        rows = m["rows"][prec]
        assert len(rows) == 16
        assert rows[0][0] <= b1, (prec, "pass 1", rows[0][0])
        worst = max(r[0] for r in rows)
        worst_rms = max(r[1] for r in rows)
        assert worst <= bmax, (prec, "worst max rel", worst)
        assert worst_rms <= brms, (prec, "worst RMS rel", worst_rms)
