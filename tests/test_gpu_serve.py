"""GPU: the autotuner (the serving loop is tested in test_gpu_pool_serve.py)."""
import numpy as np
import pytest
import torch

import oracle
from apsep_gb300 import Plan, autotune

pytestmark = pytest.mark.gpu


def test_autotune_table_and_tuned_plan():
    table = autotune.tune(dtype=torch.int32, classes=[14, 16], reps=1)
    assert set(table.entries) == {14, 16}
    assert all(0 <= c < autotune.num_configs() for c in table.entries.values())
    rng = np.random.default_rng(3)
    with Plan(1 << 17, torch.int32, tuning=table) as p:
        for n in (1 << 14, 1 << 16, 100003):
            a = rng.integers(0, 1 << 31, n, dtype=np.int64).astype(np.int32)
            out = p.run(torch.from_numpy(a).cuda())
            p.check()
            assert np.array_equal(out.cpu().numpy(), oracle.apse(a))
