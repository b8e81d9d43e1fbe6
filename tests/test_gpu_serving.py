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


def equal_submissions(dev, n, tris=4000, side=200, seed=9):
    """n submissions of the same size: one mesh draw each into its own target."""
    s = wl.scene_batched(dev, n_targets=n, n_draws=n, tri_lo=tris, tri_hi=tris, side_lo=side, side_hi=side, seed=seed)
    cmds, targets = [], []
    for k in range(n):
        enc = dev.create_command_encoder()
        wl.MultiScene(dev, passes=[s.passes[k]]).record(enc)
        cmds.append(enc.finish())
        targets.append([s.passes[k][:2]])
    return cmds, targets, s


def estimate(tris, side):
    """The documented per-submission estimate (include/gbr.h, GBR_ADMISSION_*)."""
    from wgpu_gb300 import _abi as A

    prims = tris + 2  # the draw's primitive slots: index count / 3 + 2
    return prims * A.ADMISSION_BYTES_PER_PRIMITIVE + side * side // 16 + 4096


def busy_submission(dev):
    """A submission that keeps the device busy for milliseconds with little memory: 2,000 large
    alpha-blended quads into a 3840x2160 Rgba16Float target (extension profile)."""
    q = wl.scene_blended_quads(dev, n_quads=2000, size_lo=400, size_hi=1024, seed=6)
    enc = dev.create_command_encoder()
    q.record(enc)
    return enc.finish(), q


def test_hbm_budget_admits_one_submission_per_launch():
    """A budget that holds the resident resources and one submission but not two: submissions that
    queue up behind a busy one run one per launch (batched_with == 1) with the same results as
    alone and the oracle; with the default budget the same stream merges."""
    from wgpu_gb300 import _abi as A

    ext = W.Profile.EXTENSION
    n, tris, side = 10, 4000, 200
    probe = W.Device(profile=ext, batch_submissions=True, tile_size=16, warps_per_tile=2)
    try:
        keep = (equal_submissions(probe, n, tris, side), busy_submission(probe))
        resident, _ = probe.memory()
    finally:
        probe.close()
    assert resident > 60 << 20  # the busy target alone holds 66 MB
    # resident + group + one estimate < budget < resident + group + two estimates
    budget = resident + A.ADMISSION_GROUP_BYTES + int(1.5 * estimate(tris, side))
    results = {}
    for name, kw in (("tight", dict(hbm_budget_bytes=budget)), ("default", {})):
        dev = W.Device(profile=ext, batch_submissions=True, tile_size=16, warps_per_tile=2, **kw)
        try:
            cmds, targets, keep = equal_submissions(dev, n, tris, side)
            busy, keep_busy = busy_submission(dev)
            assert dev.memory()[0] == resident
            h = dev.queue.submit([busy])
            subs = [dev.queue.submit([c]) for c in cmds]  # they queue while the busy one runs
            dev.poll(True, subs[-1])
            dev.poll(True, h)
            results[name] = ([dev.submission_stats(i) for i in subs], read_all(dev, targets))
        finally:
            dev.close()
    tight_stats, tight_frames = results["tight"]
    assert all(s.batched_with == 1 for s in tight_stats), [s.batched_with for s in tight_stats]
    assert max(s.batched_with for s in results["default"][0]) > 1, "the default budget should merge"
    assert_same_targets(tight_frames, results["default"][1], "one per launch vs merged")

    alone = W.Device(profile=ext, tile_size=16, warps_per_tile=2)
    orc = oracle_device.device(profile=ext, threads=8)
    try:
        for dev, what in ((alone, "alone"), (orc, "oracle")):
            cmds, targets, keep = equal_submissions(dev, n, tris, side)
            frags = []
            for c in cmds:
                i = dev.queue.submit([c])
                dev.poll(True, i)
                frags.append(dev.submission_stats(i).fragments_shaded)
            assert_same_targets(tight_frames, read_all(dev, targets), f"budgeted vs {what}")
            assert [s.fragments_shaded for s in tight_stats] == frags
    finally:
        alone.close()


def test_budget_below_resident_fails_with_out_of_memory():
    """Resources alone above the budget: a submission fails with OUT_OF_MEMORY, as documented."""
    dev = W.Device(batch_submissions=True, hbm_budget_bytes=1 << 20)
    try:
        s = wl.scene_colored_sphere(dev, 512, 512)
        with pytest.raises(W.GbrError) as e:
            s.render()
        assert e.value.status == -2
    finally:
        dev.close()
