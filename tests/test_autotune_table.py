"""The autotuner's table (host logic, no GPU): nearest size class, per key
type entries, JSON round trip with the recorded timings."""
import pytest

torch = pytest.importorskip("torch")

from apsep_gb300.autotune import Table, size_class  # noqa: E402


def test_nearest_class_and_key_types():
    t = Table({14: 4, 20: 2, 25: 0}, "GB300", by_dtype={"float32": {14: 5, 25: 2}},
              timings={"int32": {"14": {"0": 14.0, "4": 11.3}}})
    assert size_class(1 << 20) == 20 and size_class((1 << 20) + 5) == 20 and size_class(0) == 0
    assert t.config_for(1 << 14) == 4
    assert t.config_for(1 << 17) == 4          # nearest class 14 (ties go to the lower one)
    assert t.config_for(1 << 22) == 2 and t.config_for(1 << 30) == 0
    assert t.config_for(1 << 14, torch.int32) == 4
    assert t.config_for(1 << 14, torch.float32) == 5
    assert t.config_for(1 << 24, torch.float32) == 2
    r = Table.from_json(t.to_json())
    assert r.entries == t.entries and r.by_dtype == t.by_dtype and r.timings == t.timings
    assert Table({}).config_for(100) is None
