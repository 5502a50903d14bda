"""The benchmark's roofline arithmetic without a GPU: algorithmic bytes per point and step
of each storage kind and RK form (FP32: 624 B in form 0, 516 B in form 1; 2-byte
registers: 336 / 282 B; PML slab points 384 / 312 B), and the DRAM/algorithmic traffic
ratios read from the committed ncu summaries (FP32 in both forms, BF16 in form 1)."""
import os
import re
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_algorithmic_bytes_per_point_and_step():
    assert bench.bytes_pt_step("fp32", 0) == 624 and bench.bytes_pt_step("fp32", 1) == 516
    for st in ("bf16", "fp16"):
        assert bench.bytes_pt_step(st, 0) == 336 and bench.bytes_pt_step(st, 1) == 282
    assert bench.bytes_pml_pt_step(0) == 384 and bench.bytes_pml_pt_step(1) == 312


def test_traffic_ratios_come_from_the_profiles():
    def ratio(name, key):
        text = open(os.path.join(ROOT, "profiles", name)).read()
        return float(re.search(key + r":\s*([0-9.]+)", text).group(1))

    assert bench.ncu_traffic_ratio(1, "fp32") == ratio("stage_batch_kernel_c2.md", "dram_traffic_over_algorithmic")
    assert bench.ncu_traffic_ratio(0, "fp32") == ratio("stage_batch_kernel_c2.md",
                                                       "dram_traffic_over_algorithmic_form0")
    assert bench.ncu_traffic_ratio(1, "bf16") == ratio("stage_batch_kernel_bf16_c2.md",
                                                       "dram_traffic_over_algorithmic")
    assert bench.ncu_traffic_ratio(0, "bf16") is None
    for st in ("fp32", "bf16"):
        r = bench.ncu_traffic_ratio(1, st)
        assert 1.0 <= r < 1.5, (st, r)
