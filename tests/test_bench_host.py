"""Host-side logic of bench.py (no GPU): the ERI roofline arithmetic."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_eri_roofline_combines_kinds(bench):
    fp64, fp32 = 1.25e12, 73.2e12
    # two steps; kinds: double-float (2xx), FP32 (1xx), FP32 tail (3xx)
    sweep = {254: [20.0, 2 * 4e9, 2], 153: [2.0, 2 * 1e9, 2], 354: [1.0, 2 * 5e8, 2]}
    r = bench.eri_roofline(sweep, [10.0, 10.0], fp64, fp32, 20.0, "ch_chain")
    t_star = 4e9 / (fp32 / 2 * 3 / 16) + 1e9 / (fp32 / 2 * 3 / 2) + 5e8 / (fp32 / 2 * 3 / 2)
    assert r["frac"] == pytest.approx(t_star / 10e-3)
    assert r["achieved"] == pytest.approx(5.5e9 / 10e-3 / 1e12)
    assert r["achieved"] / r["peak"] == pytest.approx(r["frac"])
    assert r["share_of_step"] == pytest.approx(0.5)
    assert r["longest_launch"]["class"] == "(d d|d p) double-float"
    assert r["traffic"] == bench.PROFILED_TRAFFIC.get(("ch_chain", 254))
    assert r["flops_per_step"]["fp32 tail"] == pytest.approx(5e8)


def test_block_roofline_sums_kinds(bench):
    fp64, fp32 = 1.25e12, 73.2e12
    stats = {"eri_flops": {"fp64": 0.0, "fp32": 4e12, "df64": 5e11},
             "transform_flops": {"fp64": 0.0, "fp32": 2e11, "df64": 3.6e11}, "chunks": 139, "launches": 2616}
    r = bench.block_roofline(stats, [900.0, 900.0], fp64, fp32, 1000.0)
    t_star = 4e12 / (fp32 / 2 * 3 / 2) + 5e11 / (fp32 / 2 * 3 / 16) + 2e11 / fp32 + 3.6e11 / (fp32 / 12)
    assert r["frac"] == pytest.approx(t_star / 0.9)
    assert r["achieved"] == pytest.approx((4e12 + 5e11 + 2e11 + 3.6e11) / 0.9 / 1e12)
    assert r["share_of_step"] == pytest.approx(0.9)
    assert r["traffic"] == bench.PROFILED_TRAFFIC[("lif_cluster", "transform_df64")]
    assert r["flops_per_step"]["transform_df64"] == pytest.approx(3.6e11)


def test_eri_roofline_fp64_only(bench):
    r = bench.eri_roofline({53: [30.0, 3e10, 3]}, [10.0, 10.0, 10.0], 1.25e12, 73.2e12, 12.0, "water_vshf")
    assert r["frac"] == pytest.approx(1e10 / (1.25e12 / 2 * 3 / 2) / 10e-3)
    assert r["traffic"] is None
