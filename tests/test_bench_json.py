"""bench.py's JSON helpers on the CPU: the LU-solve flop count, the roofline
entry of the dominant kernel class (HBM-bound classes against the measured
copy bandwidth, the FP64 trailing update against the DFMA rate measured in
the run, the panel with its latency limiter) and the kernel-class breakdown."""
import math

import bench


def _cls(ms_step, gbs, tflops, alg_bytes, alg_flops, ms_span, share):
    return {"ms_per_step": ms_step, "achieved_gbs": gbs, "achieved_tflops": tflops,
            "alg_bytes_per_span": alg_bytes, "alg_flops_per_span": alg_flops,
            "ms_per_span": ms_span, "share_of_step": share}


def test_lu_solve_flops():
    n, r = 8192, 1
    assert bench.lu_solve_flops(n, r) == 2.0 * n ** 3 / 3 + 2.0 * n * n * r


def test_panel_roofline_names_its_limiter():
    k = {"panel": _cls(22.4, 12.0, 0.1, 2113536.0, 1.68e7, 0.1747, 0.77),
         "residual": _cls(1.26, 3400.0, 0.85, 5.4e8, 1.3e8, 0.157, 0.04)}
    r = bench.dominant_roofline(k, mixed=True)
    assert r["class"] == "panel" and r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert math.isclose(r["frac"], round(12.0 / r["peak"], 4))
    assert r["alg_per_launch"] == 2113536.0 and r["ms_per_launch"] == 0.1747
    assert r["traffic"] == 2113536.0 * bench.NCU_TRAFFIC_PER_ALG_BYTE["panel"]
    assert r["limiter"].startswith("latency: 64 sequential pivot decisions per launch")
    assert "2.73 us each" in r["limiter"]


def test_fp64_update_roofline_is_dfma_bound():
    k = {"trailing_update": _cls(300.0, 100.0, 1.0, 1e9, 1e12, 2.0, 0.85),
         "panel": _cls(20.0, 10.0, 0.1, 1e6, 1e7, 0.09, 0.06)}
    bench.FP64_PEAK.update({"tflops": 1.25, "source": "test"})
    r = bench.dominant_roofline(k, mixed=False)
    assert r["bound"] == "fp64" and r["unit"] == "TFLOP/s"
    assert r["peak"] == 1.25 and r["frac"] == round(1.0 / 1.25, 4)
    assert "limiter" not in r
    # the FP64 panel is 32 columns wide
    k["panel"]["ms_per_step"] = 400.0
    r = bench.dominant_roofline(k, mixed=False)
    assert r["limiter"].startswith("latency: 32 sequential pivot decisions")


def test_empty_breakdown_has_no_roofline():
    assert bench.dominant_roofline({}, mixed=True) is None


def test_fp64_roofline_uses_the_measured_peak():
    bench.FP64_PEAK.update({"tflops": 1.2, "source": "test"})
    r = bench.fp64_roofline(0.9)
    assert r == {"bound": "fp64", "achieved": 0.9, "peak": 1.2, "unit": "TFLOP/s", "frac": 0.75,
                 "peak_source": "test"}
    bench.FP64_PEAK.update({"tflops": None})
    assert bench.fp64_roofline(0.9)["frac"] is None
