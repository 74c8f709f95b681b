"""The bench's clock record: nvidia-smi samples are kept only inside the timed region."""
import datetime

import bench


def _line(ts, sm, reasons=("Not Active",) * 4):
    stamp = datetime.datetime.fromtimestamp(ts).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
    return ", ".join([stamp, "0", str(sm), "2070", "850.00", "0x0", *reasons])


def test_samples_outside_region_dropped():
    t0 = 1_800_000_000.0
    lines = [_line(t0 - 0.4, 345), _line(t0 + 0.1, 2070), _line(t0 + 0.3, 2055), _line(t0 + 0.5, 2070),
             _line(t0 + 1.4, 345)]
    c = bench.ClockSampler.parse(lines, t0, t0 + 1.0)
    assert c["samples"] == 3 and c["samples_in_region"] == 3
    assert c["sm_mhz"] == 2070 and c["sm_max_mhz"] == 2070 and c["reasons"] == []


def test_reasons_collected_and_fallback_to_all_samples():
    t0 = 1_800_000_000.0
    lines = [_line(t0 - 0.2, 1900, ("Not Active", "Not Active", "Not Active", "Active")),
             "garbage line", _line(t0 + 5.0, 2070)]
    # no sample inside a short region: every parsed sample is used
    c = bench.ClockSampler.parse(lines, t0, t0 + 0.05)
    assert c["samples"] == 2 and c["samples_in_region"] == 0
    assert c["reasons"] == ["sw_power_cap"]
    assert bench.ClockSampler.parse([], t0, t0 + 1)["reasons"] == ["unsampled"]
