"""GPU parity of the serving mode: with batch_submissions on, submissions queued while the
device is busy are merged into one launch (their tiles run in the same kernels); every
submission's target and fragment count must equal the same submission rendered alone and the
oracle, and a submission that fails on the device fails alone."""

import numpy as np
import pytest

import oracle_device
from wgpu_gb300 import api as W
from wgpu_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def build_stream(dev, n, seed=7):
    """A heavy first submission (keeps the device busy) and n small ones, each into its own
    target, recorded up front; returns (command buffers, colour/depth targets per submission)."""
    heavy = wl.scene_batched(dev, n_targets=8, n_draws=48, tri_lo=20000, tri_hi=200000, side_lo=512,
                             side_hi=1024, seed=seed)
    enc = dev.create_command_encoder()
    heavy.record(enc)
    cmds, targets = [enc.finish()], [[(c, d) for c, d, _ in heavy.passes]]
    small = wl.scene_batched(dev, n_targets=n, n_draws=2 * n, tri_lo=50, tri_hi=5000, side_lo=64, side_hi=256,
                             seed=seed + 1)
    for k in range(n):
        one = wl.MultiScene(dev, passes=[small.passes[k]])
        enc = dev.create_command_encoder()
        one.record(enc)
        cmds.append(enc.finish())
        targets.append([small.passes[k][:2]])
    return cmds, targets, (heavy, small)


def read_all(dev, targets):
    return [[(dev.read_texture(c), dev.read_texture(d)) for c, d in t] for t in targets]


def assert_same_targets(a, b, what):
    for s, (ta, tb) in enumerate(zip(a, b)):
        for t, ((ca, da), (cb, db)) in enumerate(zip(ta, tb)):
            assert (ca == cb).all(), f"{what}: submission {s} target {t}: colour differs"
            assert (da.view(np.uint32) == db.view(np.uint32)).all(), f"{what}: submission {s} target {t}: depth differs"


def test_merged_submissions_match_alone_and_oracle():
    n = 24
    served = W.Device(batch_submissions=True, tile_size=16, warps_per_tile=2)
    alone = W.Device(tile_size=16, warps_per_tile=2)
    orc = oracle_device.device(threads=8)
    try:
        cmds, targets, keep = build_stream(served, n)
        subs = [served.queue.submit([c]) for c in cmds]  # back to back: they queue behind the first
        served.poll(True, subs[-1])
        stats = [served.submission_stats(i) for i in subs]
        assert max(s.batched_with for s in stats) > 1, "no submissions were merged"
        got = read_all(served, targets)

        cmds_a, targets_a, keep_a = build_stream(alone, n)
        ref_frags = []
        for c in cmds_a:  # one at a time: no merging
            i = alone.queue.submit([c])
            alone.poll(True, i)
            ref_frags.append(alone.submission_stats(i).fragments_shaded)
        assert_same_targets(got, read_all(alone, targets_a), "merged vs alone")
        assert [s.fragments_shaded for s in stats] == ref_frags

        cmds_o, targets_o, keep_o = build_stream(orc, n)
        orc_frags = []
        for c in cmds_o:
            i = orc.queue.submit([c])
            orc.poll(True, i)
            orc_frags.append(orc.submission_stats(i).fragments_shaded)
        assert_same_targets(got, read_all(orc, targets_o), "merged vs oracle")
        assert ref_frags == orc_frags
    finally:
        served.close()
        alone.close()


def test_failing_submission_fails_alone():
    """One merged submission reads past its index buffer (a device-side validation error); the
    others in its launch still render, and the device stays usable."""
    n = 12
    dev = W.Device(batch_submissions=True, tile_size=16, warps_per_tile=2)
    ref = W.Device(tile_size=16, warps_per_tile=2)
    try:
        cmds, targets, keep = build_stream(dev, n)
        heavy, small = keep
        bad_k = 5
        # re-record submission bad_k with an index range past the end of its index buffer
        color, depth, draws = small.passes[bad_k]
        pl, groups, vbufs, ib, rng = draws[0]
        bad_draws = [(pl, groups, vbufs, ib, range(rng.start, rng.stop + 3 * 10 ** 6))] + draws[1:]
        enc = dev.create_command_encoder()
        wl.MultiScene(dev, passes=[(color, depth, bad_draws)]).record(enc)
        cmds[1 + bad_k] = enc.finish()
        subs = [dev.queue.submit([c]) for c in cmds]
        ok = []
        for k, i in enumerate(subs):
            try:
                dev.poll(True, i)
                ok.append(True)
            except W.GbrError:
                ok.append(False)
        assert ok == [k != 1 + bad_k for k in range(len(subs))], ok
        got = read_all(dev, targets)

        cmds_r, targets_r, keep_r = build_stream(ref, n)
        for k, c in enumerate(cmds_r):
            if k == 1 + bad_k:
                continue
            i = ref.queue.submit([c])
            ref.poll(True, i)
        want = read_all(ref, targets_r)
        got.pop(1 + bad_k)
        want.pop(1 + bad_k)
        assert_same_targets(got, want, "with a failing neighbour")
        # still usable
        s = wl.scene_colored_sphere(dev, 64, 64)
        s.render()
    finally:
        dev.close()
        ref.close()
