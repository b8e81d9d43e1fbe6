"""The full-size parity fixture (tests/golden/frame_digests.json) is current: the workload
generator still produces the inputs the oracle rendered, for every benchmark configuration.
(Building the scenes is cheap; rendering them is what the GPU tests and the fixture script do.)"""

import pytest

import frame_digests as fd
import oracle_device
from wgpu_gb300 import workloads as wl

FIXTURE = fd.load_fixture()


@pytest.mark.parametrize("name", sorted(wl.FULL_SIZE))
def test_fixture_inputs_match_generator(name):
    assert name in FIXTURE["configs"], f"{name} missing from the fixture: run tests/golden/make_frame_digests.py {name}"
    fx = FIXTURE["configs"][name]
    assert fx["arguments"] == wl.FULL_SIZE[name][2], "the configuration's arguments changed since the fixture was made"
    dev = oracle_device.device(profile=wl.FULL_SIZE[name][1])
    try:
        scene = wl.build_config(dev, name)
        assert fd.input_digest(scene) == fx["inputs"]
        assert len(wl.scene_targets(scene)) == len(fx["targets"])
    finally:
        dev.close()
    assert fx["fragments"] > 0
