"""Comparison of a CUDA frame (through the C ABI) with the CPU oracle."""
import numpy as np

HDR_TOL = 2.0 ** -10  # linear HDR radiance, max abs


def sector_entries(raw, cap):
    counter = int(raw[:8].view(np.uint64)[0])
    count, total = counter >> 32, counter & 0xFFFFFFFF
    n = min(count, cap)
    vals = raw[8:8 + 8 * n].view(np.uint32).reshape(n, 2)
    return counter, vals


def draw_lists(draw_raw, refs_raw, md):
    cnt = draw_raw[:8].view(np.uint32)
    nop, nal = int(cnt[0]), int(cnt[1])
    dc = draw_raw[8:8 + 16 * 2 * md].view(np.uint32).reshape(2 * md, 4)
    rf = refs_raw[:2 * md * 8].view(np.uint32).reshape(2 * md, 2).copy()
    rf[:, 1] &= 0xFFFF  # MeshletReference padding bytes are unspecified
    a, b = min(nop, md), min(nal, md)
    sel = np.r_[0:a, md:md + b]
    return (nop, nal), dc[sel], rf[sel]


def compare_views(r, fr, views, md, cap, errors):
    for v in views:
        gc, gv = sector_entries(r.prefix_sector(v), cap)
        oc, ov = sector_entries(fr.sector(v), cap)
        if gc != oc:
            errors.append("view %d: prefix counter gpu %#x oracle %#x" % (v, gc, oc))
        elif not np.array_equal(gv, ov):
            bad = np.nonzero((gv != ov).any(1))[0]
            errors.append("view %d: %d prefix entries differ (first %d)" % (v, len(bad), bad[0]))
        gn, gd, gr = draw_lists(r.draw_section(v), r.meshlet_references(v), md)
        on, od, orf = draw_lists(fr.draw_section(v), fr.meshlet_references(v), md)
        if gn != on:
            errors.append("view %d: draw counts gpu %s oracle %s" % (v, gn, on))
            continue
        if not np.array_equal(gr, orf):
            errors.append("view %d: %d meshlet references differ" % (v, int((gr != orf).any(1).sum())))
        if not np.array_equal(gd, od):
            errors.append("view %d: %d draw commands differ" % (v, int((gd != od).any(1).sum())))


def compare_frame(r, fr, md, cap, check_shadows=True, check_hdr=True):
    """Returns (errors, stats).  Bit-exact: prefix sectors, visible lists,
    draw commands, visibility (IDs + depth), MiscStorage, shadow maps;
    HDR within HDR_TOL."""
    errors, stats = [], {}
    views = range(5) if check_shadows else range(1)
    compare_views(r, fr, views, md, cap, errors)
    gv, ov = r.visibility(), fr.vis
    diff = gv != ov
    stats["vis_pixels_differ"] = int(diff.sum())
    stats["covered"] = int(((ov >> np.uint64(32)) != 0).sum())
    if diff.any():
        ys, xs = np.nonzero(diff)
        errors.append("visibility: %d pixels differ, first (%d,%d) gpu %#x oracle %#x" % (
            len(ys), xs[0], ys[0], int(gv[ys[0], xs[0]]), int(ov[ys[0], xs[0]])))
    if check_shadows:
        gm, om = r.misc(), fr.misc
        if not np.array_equal(gm, om):
            g32, o32 = gm.view(np.uint32), om.view(np.uint32)
            nan_ok = np.isnan(gm.view(np.float32)) & np.isnan(om.view(np.float32))
            bad = (g32 != o32) & ~nan_ok
            if bad.any():
                errors.append("misc storage: %d words differ (first word %d)" % (int(bad.sum()), int(np.nonzero(bad)[0][0])))
        gs, os_ = r.shadow_maps(), fr.shadow
        sd = gs.view(np.uint32) != os_.view(np.uint32)
        stats["shadow_texels_differ"] = int(sd.sum())
        stats["shadow_written"] = int((os_ < 1.0).sum())
        if sd.any():
            errors.append("shadow maps: %d texels differ" % int(sd.sum()))
    if check_hdr:
        gh, oh = r.hdr(), fr.hdr
        d = np.abs(gh.astype(np.float64) - oh.astype(np.float64))
        stats["hdr_max_abs"] = float(np.nanmax(d)) if d.size else 0.0
        if not (stats["hdr_max_abs"] <= HDR_TOL) or np.isnan(gh).any() != np.isnan(oh).any():
            errors.append("hdr: max abs diff %g > %g" % (stats["hdr_max_abs"], HDR_TOL))
    return errors, stats
