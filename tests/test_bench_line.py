"""The bench line's roofline entry, computed on the CPU from the committed ncu
figures (profiles/roofline_inputs.json) with made-up event times: it leads
with what binds the traversal kernel, keeps the contract's algorithmic-byte
fraction, and carries the any-hit kernel and the LBVH build (whose launch
count comes from the committed launch list)."""
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    sys.path.insert(0, ROOT)
    import bench as b
    return b


def test_roofline_block_from_committed_inputs(bench):
    peak = 6692.0
    closest_ms, anyhit_ms, build_ms = 3.37, 3.97, 0.203
    achieved = bench.BYTES_PER_RAY * 4194304 / (closest_ms / 1e3) / 1e9
    r = bench.roofline_block("bvh8_q8", achieved, peak, "measured", closest_ms, anyhit_ms, build_ms)
    json.dumps(r)  # the entry must serialise into the JSON line
    assert list(r)[0] == "binding"
    b = r["binding"]
    assert b["resource"] == "instruction issue"
    assert 0 < b["issue_active"] <= 1 and 0 < b["threads_per_warp_instruction"] <= 32
    assert 0 < b["dram_frac_of_peak"] < 1 and 0 < b["l2_frac_of_peak"] < 1
    assert r["frac"] == pytest.approx(achieved / peak)
    assert r["traffic"] > 0 and r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert r["anyhit"]["kernel_ms"] == anyhit_ms and r["anyhit"]["traffic"] > 0
    with open(os.path.join(ROOT, "profiles", "roofline_inputs.json")) as f:
        inputs = json.load(f)
    build = r["build"]
    assert build["kernel"].startswith("LBVH build (%d launches)" % inputs["build"]["launches"])
    alg = bench.BUILD_BYTES_PER_TRI * inputs["build"]["triangles"]
    assert build["achieved"] == pytest.approx(alg / (build_ms / 1e3) / 1e9)
    assert build["traffic"] == inputs["build"]["dram_bytes_read"] + inputs["build"]["dram_bytes_write"]


def test_roofline_block_of_an_uncaptured_layout(bench):
    # the ncu captures are of the 8-wide kernels: another layout reports the
    # contract's figures without a binding entry
    r = bench.roofline_block("bvh2", 1000.0, 6692.0, "measured", 6.0, 7.0, 0.2)
    assert "binding" not in r and r["traffic"] is None and r["frac"] == pytest.approx(1000.0 / 6692.0)
