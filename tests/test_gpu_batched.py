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


def _check_batched_against_oracle(lh, oracle, r, scene, probes, n, md, cap):
    """Every view of a batched frame against the oracle: the main view and
    the 4 cascades (prefix sectors, draw lists, visibility, shadow maps,
    MiscStorage, HDR within 2^-10) from the oracle's plain frame, and each
    probe (prefix sector, draw lists and commands, visibility) from the
    oracle rendering that probe as its main view."""
    errors = []
    fr = oracle.run_scene(scene, shadow_size=scene.desc.shadow_size, max_instances=cap, max_draws=md)
    # GPU batched view order: main, probes 1..n, cascades n+1..n+4; oracle: main, cascades 1..4
    for gv, ov in [(0, 0)] + [(1 + n + k, 1 + k) for k in range(4)]:
        gc, gvals = sector_entries(r.prefix_sector(gv), cap)
        oc, ovals = sector_entries(fr.sector(ov), cap)
        if gc != oc or not np.array_equal(gvals, ovals):
            errors.append("view %d: prefix sector differs" % gv)
        gn, gd, gr = draw_lists(r.draw_section(gv), r.meshlet_references(gv), md)
        on, od, orf = draw_lists(fr.draw_section(ov), fr.meshlet_references(ov), md)
        gd = gd.copy()
        gd[:, 3] -= (gv - ov) * 2 * md  # firstInstance counts from the view's reference section
        if gn != on or not np.array_equal(gr, orf) or not np.array_equal(gd, od):
            errors.append("view %d: draw lists differ (%s vs %s)" % (gv, gn, on))
    if not np.array_equal(r.visibility(), fr.vis):
        errors.append("main visibility: %d pixels differ" % int((r.visibility() != fr.vis).sum()))
    if not np.array_equal(r.shadow_maps().view(np.uint32), fr.shadow.view(np.uint32)):
        errors.append("shadow maps differ")
    gm, om = r.misc().view(np.uint32), fr.misc.view(np.uint32)
    nan_ok = np.isnan(r.misc().view(np.float32)) & np.isnan(fr.misc.view(np.float32))
    if ((gm != om) & ~nan_ok).any():
        errors.append("MiscStorage differs")
    hd = np.abs(r.hdr().astype(np.float64) - fr.hdr.astype(np.float64))
    if not float(np.nanmax(hd)) <= 2.0 ** -10:
        errors.append("hdr max abs %g" % float(np.nanmax(hd)))
    pv = r.probe_visibility(probes, n)
    covered = 0
    for p in range(n):
        fp = oracle.run_scene(scene, shadow_size=64, max_instances=cap, max_draws=md, uniforms=probes[p],
                              stages=oracle.STAGE_CULL | oracle.STAGE_RASTER)
        if not np.array_equal(pv[p], fp.vis):
            errors.append("probe %d visibility: %d pixels differ" % (p, int((pv[p] != fp.vis).sum())))
        gc, gvals = sector_entries(r.prefix_sector(1 + p), cap)
        oc, ovals = sector_entries(fp.sector(0), cap)
        if gc != oc or not np.array_equal(gvals, ovals):
            errors.append("probe %d prefix sector differs" % p)
        gn, gd, gr = draw_lists(r.draw_section(1 + p), r.meshlet_references(1 + p), md)
        on, od, orf = draw_lists(fp.draw_section(0), fp.meshlet_references(0), md)
        gd = gd.copy()
        gd[:, 3] -= (1 + p) * 2 * md
        if gn != on or not np.array_equal(gr, orf) or not np.array_equal(gd, od):
            errors.append("probe %d draw lists differ (%s vs %s)" % (p, gn, on))
        covered += int(((pv[p] >> np.uint64(32)) != 0).sum())
    return errors, covered


def test_full_batched_workload_matches_oracle(native, oracle):
    """The benched batched workload at full size -- the large scene's 1920 x
    1080 main view, its 32 probes of 64^2 to 512^2 and 4 cascades at 2048^2
    fitted from the depth reduction -- under the per-stage schedule, the
    persistent launch and the CUDA-graph replay: every view bit exact
    against the oracle."""
    lh = native
    scene = lh.Scene(3).upload(0)
    d = scene.desc
    probes, n = scene.probe_uniforms()
    assert (n, d.shadow_size, d.width, d.height) == (32, 2048, 1920, 1080)
    sizes = [lh.uniforms_fields(probes[p])["window_size"] for p in range(n)]
    assert min(min(s) for s in sizes) >= 64 and max(max(s) for s in sizes) <= 512
    px = sum((w * h + 31) // 32 * 32 for w, h in sizes)
    md, cap = 2000000, max(1024, d.n_instances)  # some probes see more than 200k meshlets
    r = lh.Renderer(lh.Config(width=d.width, height=d.height, shadow_size=d.shadow_size, max_instances=cap,
                              max_draws=md, max_probes=n, max_probe_pixels=px))
    r.set_scene(scene)
    u = scene.uniforms
    for name, sched, graph in (("per-stage", lh.SCHEDULE_PER_STAGE, False),
                               ("persistent", lh.SCHEDULE_PERSISTENT, False),
                               ("per-stage graph", lh.SCHEDULE_PER_STAGE, True)):
        r.set_tuning(schedule=sched)
        if graph:
            r.frame_graph(u, probes, n)
            r.frame_graph(u, probes, n)  # captured on the first call, replayed on the second
        else:
            r.frame_batched(u, probes, n)
        st = r.status()
        assert st.flags == 0, (name, hex(st.flags))
        errors, covered = _check_batched_against_oracle(lh, oracle, r, scene, probes, n, md, cap)
        assert not errors, "%s: %s" % (name, errors[:8])
        assert covered > 0
