"""Host arithmetic of bench.py's JSON line, without a GPU: the roofline object of the dominant stage
(achieved = the work model's flops or bytes per launch over the CUDA-event time per launch; traffic =
the ncu ratio of a small capture times this run's units per launch) and the reference arm's
iteration-count label."""
import pytest

import bench

PEAKS = (6783.8, 1932.6, "measured")


def _stage(ms, launches, flops_per, bytes_per):
    return {"ms": ms, "launches": launches, "flops": flops_per * launches, "bytes": bytes_per * launches}


def test_roofline_of_the_residual_product_at_the_headline_size():
    # one refined iteration of the 1.05 deg bilayer: 16 k, 9.98 s in the sliced residual product
    n, iu = 11908, 11908 // 2 + 10
    flops = 15 * 8.0 * n * n * iu          # depth 4: 15 slice pairs, complex n x n times n x iu
    nbytes = n * iu * 16.0 * 2 + n * n * 16.0
    kernels = {"oa_gemm": _stage(9980.0, 16, flops, nbytes), "hemv": _stage(7620.0, 16 * n, 1.0, 1.0),
               "invit": _stage(4090.0, 16, 0.0, 0.0)}
    roof = bench.roofline(kernels, "fast", PEAKS)
    assert roof["kernel"] == "oa_gemm" and roof["bound"] == "tensor" and roof["unit"] == "TFLOP/s"
    assert roof["achieved"] == pytest.approx(flops / (9980.0e-3 / 16) / 1e12)
    assert roof["achieved"] == pytest.approx(162.7, abs=0.5)
    assert roof["frac"] == pytest.approx(roof["achieved"] / 1932.6)
    # traffic per launch scales with the slice-product flops (0.01628 B per flop at N = 5044)
    assert roof["traffic"] == pytest.approx(0.01628 * flops)
    assert "per algorithmic flop" in roof["traffic_source"]
    assert roof["peak_source"].startswith("measured")


def test_roofline_of_an_fp64_run_is_hbm_bound():
    n = 11908
    kernels = {"hemv": _stage(7620.0, 16 * n, 1.0, 5.0e8), "backtransform": _stage(6600.0, 16, 1e13, 1e9)}
    roof = bench.roofline(kernels, "plain", PEAKS)
    assert roof["kernel"] == "hemv" and roof["bound"] == "hbm" and roof["unit"] == "GB/s"
    assert roof["achieved"] == pytest.approx(5.0e8 / (7620.0e-3 / (16 * n)) / 1e9)
    assert roof["traffic"] == pytest.approx(1.044 * 5.0e8)
    # a stage without an ncu capture carries no traffic figure
    roof = bench.roofline({"backtransform": _stage(6600.0, 16, 1e13, 1e9)}, "plain", PEAKS)
    assert roof["traffic"] is None and roof["traffic_source"] is None


def test_roofline_without_a_throughput_stage_is_null():
    assert bench.roofline({"invit": _stage(1.0, 1, 0.0, 0.0), "bisect": _stage(1.0, 1, 0.0, 0.0)}, "fast",
                          PEAKS) is None


def test_reference_arm_labels_the_estimated_iteration_count():
    rec = bench.PLAIN_FP64_RECORDED["tbg_m31_N11908_4x4_nu+2_eps10_1.05deg"]
    assert rec["estimated"] and rec["time_to_scf_s"] == pytest.approx(rec["guess_s"] + 11 * 347.8)
    assert "FP64-equivalent" in bench._iterations_source(rec)
    assert bench._iterations_source(bench.PLAIN_FP64_RECORDED["tbg_m10_N1324_12x12_nu+2_eps10"]).startswith(
        "measured")
    assert "value is null" in bench._iterations_source(None)
