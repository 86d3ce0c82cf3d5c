"""Batched multi-view frames (main + probes + cascades): every schedule (one
launch per stage, one persistent launch, one launch per view) and the CUDA
graph replay give the same bits, and each probe view matches the oracle
rendering that probe as its main view."""
import numpy as np
import pytest

from tests.parity import compare_frame, compare_views, draw_lists, sector_entries

pytestmark = pytest.mark.gpu


def _setup(lh, config=2, n_probes=6, **params):
    scene = lh.Scene(config, n_probes=n_probes, **params).upload(0)
    d = scene.desc
    probes, n = scene.probe_uniforms()
    px = sum((lh.uniforms_fields(probes[p])["window_size"][0] * lh.uniforms_fields(probes[p])["window_size"][1] + 31)
             // 32 * 32 for p in range(n))
    cfg = lh.Config(width=d.width, height=d.height, shadow_size=d.shadow_size, max_instances=max(1024, d.n_instances),
                    max_draws=200000, max_probes=max(n, 1), max_probe_pixels=max(px, 32))
    r = lh.Renderer(cfg)
    r.set_scene(scene)
    return scene, r, probes, n


def _snapshot(r, probes, n, md=200000, cap=1024):
    """Valid parts of every result: prefix entries up to the count, draw
    lists up to their counts (stale bytes past them are not results)."""
    out = {"vis": r.visibility(), "hdr": r.hdr(), "shadow": r.shadow_maps(), "misc": r.misc(),
           "probes": r.probe_visibility(probes, n)}
    for v in range(5 + n):
        c, vals = sector_entries(r.prefix_sector(v), cap)
        out["sector%d" % v] = np.concatenate([np.array([c], np.uint64).view(np.uint32), vals.reshape(-1)])
        cnt, dc, rf = draw_lists(r.draw_section(v), r.meshlet_references(v), md)
        out["draw%d" % v] = np.concatenate([np.array(cnt, np.uint32), dc.reshape(-1)])
        out["refs%d" % v] = rf
    return out


def _same(a, b):
    bad = []
    for k in a:
        if k == "probes":
            for i, (x, y) in enumerate(zip(a[k], b[k])):
                if not np.array_equal(x, y):
                    bad.append("probe %d" % i)
        elif a[k].shape != b[k].shape or not np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)):
            bad.append(k)
    return bad


def test_schedules_identical(native):
    lh = native
    scene, r, probes, n = _setup(lh, detail=0.25, n_instances=1024, width=960, height=540)
    u = scene.uniforms
    snaps = {}
    for sched in (lh.SCHEDULE_PER_STAGE, lh.SCHEDULE_PERSISTENT, lh.SCHEDULE_PER_VIEW):
        r.set_tuning(schedule=sched)
        r.frame_batched(u, probes, n)
        st = r.status()
        assert st.flags == 0, (sched, hex(st.flags))
        snaps[sched] = _snapshot(r, probes, n)
    base = snaps[lh.SCHEDULE_PER_STAGE]
    for sched in (lh.SCHEDULE_PERSISTENT, lh.SCHEDULE_PER_VIEW):
        bad = _same(base, snaps[sched])
        assert not bad, "schedule %d differs: %s" % (sched, bad)


def test_probe_views_match_oracle(native, oracle):
    lh = native
    scene, r, probes, n = _setup(lh, detail=0.25, n_instances=1024, width=960, height=540)
    r.set_tuning(schedule=lh.SCHEDULE_PERSISTENT)
    r.frame_batched(scene.uniforms, probes, n)
    # main view + cascades as in the plain frame (cascades are views 1+n .. 4+n here)
    fr = oracle.run_scene(scene, shadow_size=scene.desc.shadow_size, max_instances=1024, max_draws=200000)
    assert np.array_equal(r.visibility(), fr.vis)
    assert np.array_equal(r.shadow_maps().view(np.uint32), fr.shadow.view(np.uint32))
    pv = r.probe_visibility(probes, n)
    covered = 0
    for p in range(n):
        fp = oracle.run_scene(scene, shadow_size=64, max_instances=1024, max_draws=200000, uniforms=probes[p],
                              stages=oracle.STAGE_CULL | oracle.STAGE_RASTER)
        assert np.array_equal(pv[p], fp.vis), "probe %d visibility differs" % p
        gc, gv = sector_entries(r.prefix_sector(1 + p), 1024)
        oc, ov = sector_entries(fp.sector(0), 1024)
        assert gc == oc and np.array_equal(gv, ov), "probe %d prefix sector differs" % p
        gn, gd, gr = draw_lists(r.draw_section(1 + p), r.meshlet_references(1 + p), 200000)
        on, od, orf = draw_lists(fp.draw_section(0), fp.meshlet_references(0), 200000)
        assert gn == on and np.array_equal(gr, orf), "probe %d draw lists differ" % p
        base = (1 + p) * 2 * 200000
        gd = gd.copy()
        gd[:, 3] -= base  # firstInstance counts from the probe's reference section
        assert np.array_equal(gd, od), "probe %d draw commands differ" % p
        covered += int(((pv[p] >> np.uint64(32)) != 0).sum())
    assert covered > 0


def test_graph_replay_matches_direct(native, oracle):
    lh = native
    scene, r, probes, n = _setup(lh, config=1, n_probes=3)
    d = scene.desc
    u1 = scene.uniforms
    u2 = lh.make_uniforms((10.0, 5.0, -140.0), 1.5, 0.05, 60.0, d.width, d.height, d.n_instances)
    r.frame_batched(u2, probes, n)
    direct = _snapshot(r, probes, n)
    for u in (u1, u2):  # capture on the first call, replay with new uniforms on the second
        r.frame_graph(u, probes, n)
    replay = _snapshot(r, probes, n)
    assert not _same(direct, replay)
    fr = oracle.run_scene(scene, shadow_size=d.shadow_size, max_instances=1024, max_draws=200000, uniforms=u2)
    assert np.array_equal(replay["vis"], fr.vis)
