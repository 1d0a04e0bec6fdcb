"""CPU: the bench's roofline arithmetic and the shape of its JSON line.

The per-step algorithmic bytes follow the workload's definition: per RHS 11
transforms x (N + Next) values read and written plus the result write,
15 (N + Next) values; per DOPRI853 step 12 RHS evaluations and 72 Ntot values
of stage combinations (61 stage-input reads, 1 post-step read, 9 final reads,
1 write): 63.1 GB in FP32 at 256^3, a 9.3 ms floor at the measured copy peak.
The committed bench record (profiles/bench_256.json, the line of a run of
this bench.py on a GB300) carries every key of the line's contract."""
import importlib.util
import json
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _bench():
    spec = importlib.util.spec_from_file_location("bench_module", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_step_bytes_and_floor():
    b = _bench()
    r = b.step_roofline(10.0, 6778.3, "measured")
    n = 256
    N, Next = n ** 3, 2 * n * n * (n // 2 + 1)
    Ntot = 4 * N + 4 * Next + 1
    assert N + Next == 33_685_504 and Ntot == 134_742_017
    assert r["bytes_per_step"] == (12 * 15 * (N + Next) + 72 * Ntot) * 4 == 63_059_263_776
    assert abs(r["floor_ms_per_step"] - 9.303) < 1e-3
    assert abs(r["achieved"] - 6305.93) < 0.01 and abs(r["frac"] - 6305.93 / 6778.3) < 1e-6


def test_committed_bench_record_has_the_contract_keys():
    d = json.loads((ROOT / "profiles" / "bench_256.json").read_text())
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "gpu_launches", "e2e", "roofline", "clocks"):
        assert k in d, k
    assert d["n_gpus"] == 1 and d["warmup"] >= 3 and d["higher_is_better"] is True
    assert d["unit"] == "m*t/s" and d["value"] > 0 and d["gpu_launches"] > 0
    assert "workload" in d["config"] and "l2" in d["config"]
    rf = d["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in rf, k
    assert rf["bound"] == "hbm" and rf["unit"] == "GB/s"
    assert abs(rf["frac"] - rf["achieved"] / rf["peak"]) < 1e-9
    e = d["e2e"]
    for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"):
        assert k in e, k
    assert e["h2d_bytes_per_step"] == e["d2h_bytes_per_step"] == 16 * 134_742_017
    c = d["clocks"]
    for k in ("sm_mhz", "sm_max_mhz", "reasons"):
        assert k in c, k
    acc = d["accuracy_vs_f64"]
    assert acc["t_end"] >= 10 and acc["within_1pct"] is True and acc["gw_max_rel_diff"] < 0.01
    cpu = d["cpu_baseline"]
    for k in ("value", "unit", "cores", "kind", "sample", "ms_per_step", "dt_per_step", "gpu_dt"):
        assert k in cpu, k
    assert cpu["kind"] in ("reference", "port") and cpu["cores"] >= 1
    # the CPU arm starts from the GPU arm's state with the GPU arm's step size
    assert cpu["dt_per_step"][0] == cpu["gpu_dt"]
    assert d["f64"]["roofline"]["fp64"]["peak_source"] == "measured"


def test_f64_form_bounds():
    """The FP64 form against both of its bounds at 256^3: 126.1 GB per step
    against HBM, 1.54e11 flops against the FP64 pipe -- the pipe binds."""
    b = _bench()
    r = b.f64_roofline(274.0, 6778.3, "measured", 1.25, "measured")
    assert r["hbm"]["bytes_per_step"] == 2 * 63_059_263_776
    assert abs(r["fp64"]["flops_per_step"] - 1.5443e11) < 1e8
    assert abs(r["fp64"]["floor_ms_per_step"] - 123.5) < 0.5
    assert r["bound"] == "fp64" and r["fp64"]["frac"] > r["hbm"]["frac"]
