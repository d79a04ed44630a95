"""CPU checks of the bench's roofline arithmetic: which roof bounds a kernel
class, what `achieved` and `frac` are, and which traffic entries apply."""
import json

import bench


def _v(ms, bytes_, flops, launches=10):
    return {"ms": ms, "bytes": bytes_, "flops": flops, "launches": launches}


def test_fp64_class_is_bound_by_the_fp64_pipe():
    # 1 TFLOP in 1 s on a 1.1 TF/s FP64 pipe; its bytes would take far less at 6.8 TB/s
    e = bench.roofline_entry("gram", _v(1000.0, 1e11, 1e12), 6800.0, 1.1, {})
    assert e["bound"] == "fp64" and e["unit"] == "TFLOP/s"
    assert abs(e["achieved"] - 1.0) < 1e-12 and abs(e["frac"] - 1.0 / 1.1) < 1e-12
    assert e["avg_launch_ms"] == 100.0 and e["algorithmic_flops_per_launch"] == 1e11


def test_fp32_class_is_never_taken_for_an_fp64_one():
    # the same numbers under the FP32 class name: HBM-bound, achieved in GB/s
    e = bench.roofline_entry("gram_fp32", _v(1000.0, 1e11, 1e12), 6800.0, 1.1, {})
    assert e["bound"] == "hbm" and e["unit"] == "GB/s"
    assert abs(e["achieved"] - 100.0) < 1e-9 and abs(e["frac"] - 100.0 / 6800.0) < 1e-12


def test_tensor_class_bound_by_the_tensor_rate_only_when_slower_than_hbm():
    hbm = bench.roofline_entry("tc_gram", _v(1.0, 6.8e9, 1e9), 6800.0, 1.1, {},
                               fp64_arith=False, tf32_peak=960.0)
    assert hbm["bound"] == "hbm" and abs(hbm["frac"] - 1.0) < 1e-9
    ten = bench.roofline_entry("tc_gram", _v(1.0, 1e6, 9.6e11), 6800.0, 1.1, {},
                               fp64_arith=False, tf32_peak=960.0)
    assert ten["bound"] == "tensor" and abs(ten["frac"] - 1.0) < 1e-9


def test_traffic_entries_are_filtered_by_workload(tmp_path, monkeypatch):
    prof = tmp_path / "profiles"
    prof.mkdir()
    (prof / "traffic.json").write_text(json.dumps({
        "gram": {"bytes_per_launch": 123, "config": "c2"},
        "stencil7_fp32": {"bytes_per_launch": 456, "config": "c3"}}))
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert set(bench.load_traffic("c2")) == {"gram"}
    assert set(bench.load_traffic("c3")) == {"stencil7_fp32"}
    e = bench.roofline_entry("gram", _v(1000.0, 1e11, 1e12), 6800.0, 1.1, bench.load_traffic("c2"))
    assert e["traffic"] == 123


def test_committed_traffic_file_names_its_workloads():
    traffic = bench.load_traffic("c2")
    assert "gram" in traffic and traffic["gram"]["bytes_per_launch"] > 0


def test_nested_rayleigh_ritz_stages_stay_out_of_the_total():
    # sygv's record spans its rr_* stages and the fallback gate: counting
    # them again would inflate the total the shares are taken of
    kt = {"oz_gram": _v(30.0, 0, 0), "sygv": _v(10.0, 0, 0), "rr_tridiag": _v(4.0, 0, 0),
          "rr_bisect": _v(3.0, 0, 0), "sygv_fp64_gate": _v(0.1, 0, 0), "blas1": _v(60.0, 0, 0)}
    assert bench.nested("rr_tridiag") and bench.nested("sygv_fp64_gate")
    assert not bench.nested("sygv") and not bench.nested("blas1")
    assert bench.top_level_ms(kt) == 100.0
    assert bench.top_level_ms({}) == 1.0


def test_reference_arm_scales_by_the_recorded_fp64_iteration_count():
    assert bench.CONFIGS["c3m"]["fp64_iterations"] == 176
    assert bench.CONFIGS["c3"]["fp64_iterations"] == 565


def test_adjoint_record_keeps_its_fields_and_reports_failures(monkeypatch):
    """The derivative record beside the headline carries the forward and
    backward times of the adjoint configuration's line; a failure there
    becomes an error field instead of ending the run."""
    fake = {"config": {"workload": "w"}, "forward_ms": 100.0, "backward_ms": 25.0, "value": 125.0,
            "fwd_plus_bwd_over_fwd": 1.25, "lobpcg_iterations": 9, "adjoint_cg_iterations": 4,
            "adjoint_max_rel_residual": 1e-9, "e2e": {"value": 130.0}, "gpu_launches": 7}
    monkeypatch.setattr(bench, "measure_adjoint", lambda *a, **k: fake)
    rec = bench.adjoint_summary("c4", 1, 0, None)
    assert rec["config"] == "c4" and rec["fwd_plus_bwd_ms"] == 125.0
    assert rec["fwd_plus_bwd_over_fwd"] == 1.25 and rec["e2e_ms"] == 130.0

    def boom(*a, **k):
        raise RuntimeError("no device")
    monkeypatch.setattr(bench, "measure_adjoint", boom)
    rec = bench.adjoint_summary("c4", 1, 0, None)
    assert rec == {"config": "c4", "error": "RuntimeError: no device"}
    assert bench.CONFIGS["c3m"]["adjoint"] == "c4" and bench.CONFIGS["c4"]["kind"] == "adjoint5"
