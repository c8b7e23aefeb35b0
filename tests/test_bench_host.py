"""bench.py's host-side arithmetic, without a GPU: the roofline numerator (algorithmic
FLOPs per atom), the clock summaries of the timed region (nvidia-smi record and NVML
samples) and the extrapolation of the sampled CPU baseline to a full structure."""
import time

import numpy as np
import pytest

import bench
from quip_gb300 import models


@pytest.mark.parametrize("name, nu, expected", [
    # canonical per-atom count 2 [nu n L^2 + P L^2 + 2 D M + N^2 L^2 + 3 nu n L^2]
    ("si64", 28, 2 * (10976 + 1764 + 253000 + 3136 + 32928)),             # 0.60 MFLOP/atom
    ("sic32768", 50, 2 * (40500 + 17010 + 30256000 + 32400 + 121500)),    # 60.9 MFLOP/atom
])
def test_algorithmic_flops_per_atom(name, nu, expected):
    w = bench.WORKLOADS[name]
    total, gemm = bench.algorithmic_flops(w, nu)
    assert total == expected
    n, L, ns = w["n_max"], w["l_max"] + 1, len(w["species"])
    N = n * ns
    D = N * (N + 1) // 2 * L + 1
    assert D == models.soap_dim(n, w["l_max"], ns)
    assert gemm == 4 * D * w["M"]          # the two kernel GEMMs: K = Q X^T and G = W X


def test_clock_record_summary(tmp_path):
    """The nvidia-smi record taken during the timed region (index, clocks.sm,
    clocks.max.sm, power, active mask, hw_slowdown, hw_thermal, sw_thermal, sw_power_cap):
    median SM clock of the first GPU's rows, its maximum, and every reason seen Active."""
    rows = ["0, 2070, 2070, 900.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
            "1, 1200, 2070, 300.0, 0x0000000000000000, Active, Not Active, Not Active, Not Active",
            "0, 2055, 2070, 1380.5, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
            "0, 2070, 2070, 1101.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"]
    p = tmp_path / "clocks.csv"
    p.write_text("\n".join(rows) + "\n")
    c = bench.Clocks(str(p))
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]      # the other GPU's hw_slowdown row is not ours
    p.write_text("")
    assert s.keys() >= {"sm_mhz", "sm_max_mhz", "reasons"}
    assert bench.Clocks(str(p)).summary()["sm_mhz"] is None


def test_nvml_clock_summary():
    """The NVML samples (SM MHz, clock-event reason mask) taken during the timed region:
    median SM clock and every reason bit seen set, by name (0x4 sw_power_cap, 0x8
    hw_slowdown, 0x20 sw_thermal_slowdown, 0x40 hw_thermal_slowdown); unnamed bits (0x1
    idle) are left out.  No NVML call is made: the samples are planted."""
    c = object.__new__(bench.NvmlClocks)
    c.max_mhz, c.period = 2070.0, 0.01
    c.samples = []
    s = c.summary()
    assert s["sm_mhz"] is None and s["samples"] == 0 and s["sm_max_mhz"] == 2070.0
    c.samples = [(2070.0, 0x0), (2055.0, 0x4), (2070.0, 0x1), (1980.0, 0x4 | 0x20), (2070.0, 0x0)]
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["samples"] == 5
    assert s["reasons"] == ["sw_power_cap", "sw_thermal_slowdown"]
    assert "10 ms" in s["source"]


class _TimedOracle:
    """Stands in for the oracle: a call costs FIXED seconds plus PER seconds per centre."""
    FIXED, PER = 0.05, 0.002

    def calc(self, pos, Z, lat, pbc, mask=None, nthreads=1):
        k = len(Z) if mask is None else int(np.count_nonzero(mask))
        time.sleep(self.FIXED + self.PER * k)
        return {}


def test_cpu_baseline_spreads_the_fixed_cost_over_the_structure(monkeypatch):
    from oracle import oracle
    monkeypatch.setattr(oracle.OracleModel, "from_xml", staticmethod(lambda path: _TimedOracle()))
    w = dict(bench.WORKLOADS["sic32768"], name="sic32768")
    at = models.Atoms(np.full(1000, 14), np.zeros((1000, 3)), lattice=np.eye(3) * 50.0)
    cb = bench.cpu_reference(w, at, "unused.xml", steps=3, warmup=1, sample_atoms=40)
    n, fx, per = 1000, _TimedOracle.FIXED, _TimedOracle.PER
    assert cb["seconds_fixed"] == pytest.approx(fx, rel=0.5)
    assert cb["seconds_per_centre"] == pytest.approx(per, rel=0.3)
    # the full structure's rate, not the sample's (40 / (fixed + 40 per) would be ~1.5x lower)
    assert cb["value"] == pytest.approx(n / (fx + n * per), rel=0.2)
    assert cb["value"] > 1.2 * 40 / (fx + 40 * per)
    assert set(bench.CPU_KEYS) <= set(cb) | {"seconds_fixed", "seconds_per_centre"}
    assert cb["kind"] == "port" and "no centres" in cb["sample"]
