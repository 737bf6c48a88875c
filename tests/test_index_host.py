"""Host-side rejection of out-of-range collider indices (no GPU needed): the
Python layer raises IndexError before anything is copied to the device."""
import numpy as np
import pytest
import torch

from distance3d_gb300.store import as_index


@pytest.mark.parametrize("idx", [[0, 1, 10], np.array([3, -1], np.int64), torch.tensor([5, 2**31 + 4]),
                                 np.array([2**40], np.int64)])
def test_out_of_range_host_indices_raise(idx):
    with pytest.raises(IndexError, match=r"out of range \[0, 10\)"):
        as_index(idx, "cpu", 10)


def test_in_range_host_indices_pass():
    t = as_index(np.array([0, 9, 4], np.int64), "cpu", 10)
    assert t.dtype == torch.int32 and t.tolist() == [0, 9, 4]
    assert as_index([], "cpu", 0).numel() == 0
    with pytest.raises(TypeError):
        as_index(np.array([0.5]), "cpu", 10)
