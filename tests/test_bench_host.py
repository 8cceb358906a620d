"""bench.py's host logic, without a GPU: the timed window that carries the density
re-initialisation steps, the algorithmic byte counts behind roofline.achieved, the launch
count behind gpu_launches, and the clock summary that marks a throttled run."""
import importlib.util
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("steps", [1, 2, 20, 29, 30, 31, 100, 3000])
@pytest.mark.parametrize("warmup", [0, 3, 5, 40])
def test_timed_window_ends_on_a_reinit_step_and_holds_its_share(bench, steps, warmup):
    first, s0 = bench.timed_window(steps, warmup, 30)
    assert first >= 1
    assert s0 - first == warmup
    assert (s0 + steps - 1) % 30 == 0  # the window ends on a re-initialisation step
    assert bench.reinit_count(s0, steps, 30) == -(-steps // 30)


def test_timed_window_without_reinit(bench):
    assert bench.timed_window(20, 5, 0) == (1, 6)
    assert bench.reinit_count(6, 20, 0) == 0


def test_algorithmic_bytes_of_the_bench_scene(bench):
    from ethersph_gb300 import scenes
    s = scenes.natural_convection_2d(n=32)
    nf, nw = s.n_fluid, s.n_wall
    e = 25.62  # list entries a particle
    lst = 4 + 4 * e
    # continuity: fa fb cell scene rho m | rhoc p c P vol fb | the list it records
    assert bench.algorithmic_bytes(s, "fp32c", "continuity", e) == pytest.approx(nf * (56 + 56 + lst))
    # momentum: fa fb fc c cell scene, x v T rhoc | x' v' T' rho' key slot | the list; walls' shadows
    assert bench.algorithmic_bytes(s, "fp32c", "momentum", e) == pytest.approx(nf * (112 + 56 + lst) + nw * 48)
    # without the list the walks read no list bytes
    assert bench.algorithmic_bytes(s, "fp32c", "momentum") == nf * 168 + nw * 48
    assert bench.algorithmic_bytes(s, "fp64", "continuity") == nf * 84
    assert bench.algorithmic_bytes(s, "fp64", "momentum") == nf * 156 + nw * 76


def test_scan_launches_follow_the_grid(bench):
    assert bench.scan_launches(16_384) == 1
    assert bench.scan_launches(71_824) == 1   # the bench scene: one down-sweep over pre-summed tiles
    assert bench.scan_launches(262_144) == 1
    assert bench.scan_launches(262_145) == 3


def test_clock_summary_marks_throttling(bench):
    c = bench.ClockSampler()
    c.samples = [["0", "2070", "2070", "800.0", "0x0", "Not Active", "Not Active", "Not Active", "Not Active"],
                 ["0", "2055", "2070", "1390.0", "0x4", "Not Active", "Not Active", "Not Active", "Active"],
                 ["0", "2070", "2070", "900.0", "0x0", "Not Active", "Not Active", "Not Active", "Not Active"]]
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]
    c.samples.append(["0", "1400", "2070", "700.0", "0x40", "Not Active", "Active", "Not Active", "Not Active"])
    assert "hw_thermal_slowdown" in c.summary()["reasons"]
    assert bench.ClockSampler().summary()["reasons"] == ["unsampled"]
