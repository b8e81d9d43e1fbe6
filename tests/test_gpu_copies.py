"""Encoder copies and clears on the GPU (extension profile): every resource the commands touch,
including a copy ordered between two render passes, bit for bit with the oracle; the parity
profile rejects them as the reference does (todo!, command.rs:37-115)."""

import numpy as np
import pytest

import oracle_device
import scenes
from wgpu_gb300 import _abi as A
from wgpu_gb300 import api as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("graphs", [False, True])
def test_copies_match_oracle(graphs):
    dev = W.Device(profile=W.Profile.EXTENSION, use_graphs=graphs)
    try:
        g = scenes.copy_scenario(dev)
    finally:
        dev.close()
    o = scenes.copy_scenario(oracle_device.device(profile=W.Profile.EXTENSION))
    for k in ("B", "C", "X", "Y"):
        assert np.array_equal(g[k], o[k]), k
    for k in ("T1", "T2"):
        for m in range(3):
            assert np.array_equal(g[k][m], o[k][m]), (k, m)


def test_parity_profile_rejects_copies():
    dev = W.Device()
    try:
        A_ = dev.create_buffer_init(np.zeros(1024, np.uint8))
        B = dev.create_buffer_init(np.zeros(1024, np.uint8))
        enc = dev.create_command_encoder()
        enc.copy_buffer_to_buffer(A_, 0, B, 0, 64)
        with pytest.raises(W.GbrError) as e:
            dev.queue.submit([enc.finish()])
        assert e.value.status == A.ERR_UNSUPPORTED and "todo" in e.value.message
    finally:
        dev.close()
