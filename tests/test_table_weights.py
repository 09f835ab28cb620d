"""FlowTable.count_once_weights: 1 / (rows of the row's group), so that each
group's count term enters a training loss once."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from neutrinotelescopes_gb300.tables import FlowTable  # noqa: E402


def test_count_once_weights():
    rg = torch.tensor([2, 0, 0, 2, 0, 3], dtype=torch.int32)
    n = rg.numel()
    t = FlowTable(torch.zeros((n, 5)), torch.zeros(n), torch.zeros(n), torch.ones(n, dtype=torch.int32),
                  torch.zeros((5, 5)), torch.zeros(5, dtype=torch.float64), torch.zeros(5, dtype=torch.int64),
                  row_group=rg)
    w = t.count_once_weights().numpy()
    np.testing.assert_allclose(w, [1 / 2, 1 / 3, 1 / 3, 1 / 2, 1 / 3, 1.0], rtol=1e-7)
    # every group's weights sum to one
    np.testing.assert_allclose(np.bincount(rg.numpy(), weights=w), [1.0, 0.0, 1.0, 1.0])
    with pytest.raises(ValueError):
        FlowTable(t.cond, t.tres, t.nhits, t.has_time, t.group_cond, t.group_expec, t.group_count).count_once_weights()
