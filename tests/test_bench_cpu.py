"""bench.py's roofline record (host logic, no GPU): which roof binds each
kernel, and counters that are reported only for the kernel sources they were
captured on."""
import bench


def _kern():
    return {"face_flux": {"ms": 0.12, "bytes": 53.3e6, "gbs": 444.0},
            "gradients": {"ms": 0.115, "bytes": 71.2e6, "gbs": 619.0},
            "ilu0_apply": {"ms": 0.15, "bytes": 77.9e6, "gbs": 519.0}}


def test_residual_kernels_against_the_fp64_roof():
    dfma = 6.27e11
    r = bench.roofline("face_flux", _kern(), 314880, 6760.0, "measured", dfma)
    cnt = bench.NCU_COUNTS["face_flux"]
    if bench.NCU_COUNTS["sources"] == bench.kernel_sources_digest():
        assert r["bound"] == "fp64" and r["unit"] == "TFLOP/s"
        assert abs(r["achieved"] - cnt["fp64_flop"] / 0.12e-3 / 1e12) <= 1e-9
        assert abs(r["frac"] - cnt["fp64_flop"] / 0.12e-3 / (2 * dfma)) <= 1e-12
        assert r["traffic"] == cnt["dram_bytes"] and r["hbm"]["frac"] == 444.0 / 6760.0
    else:  # counters of other sources are not reported
        assert r["bound"] == "hbm" and r["traffic"] is None and "note" in r


def test_sweep_against_hbm_with_its_own_traffic():
    r = bench.roofline("ilu0_apply", _kern(), 314880, 6760.0, "measured", 6.27e11)
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["frac"] == 519.0 / 6760.0
    fresh = bench.NCU_ILU["sources"] == bench.kernel_sources_digest(bench.ILU_SOURCES)
    assert r["traffic"] == (bench.NCU_ILU["dram_bytes"] if fresh else None)


def test_stale_counters_are_not_reported(monkeypatch):
    monkeypatch.setitem(bench.NCU_COUNTS, "sources", "0" * 16)
    monkeypatch.setitem(bench.NCU_ILU, "sources", "0" * 16)
    r = bench.roofline("face_flux", _kern(), 314880, 6760.0, "measured", 6.27e11)
    assert r["bound"] == "hbm" and r["traffic"] is None
    r = bench.roofline("ilu0_apply", _kern(), 314880, 6760.0, "measured", 6.27e11)
    assert r["traffic"] is None


def test_both_arms_name_the_same_workload():
    a, b = bench.workload_config(1), bench.workload_config(1)
    assert a == b and a["workload"] == bench.WORKLOAD and a["cells"] == 183296 and a["faces"] == 314880
    assert bench.workload_config(2)["parallelism"] == "replicas2"
