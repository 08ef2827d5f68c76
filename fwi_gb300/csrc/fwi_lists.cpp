// Grid layout and work lists of the FWI time-step kernels (see fwi_lists.h).
#include "fwi_lists.h"

#include <algorithm>
#include <map>
#include <utility>

namespace fwi {

Layout make_layout(int ny, int nx, int acc, int dpml) {
    Layout l;
    l.ny = ny;
    l.nx = nx;
    l.dn = dpml + 2 * acc;
    l.acc = acc;
    l.nyt = 2 * l.dn + ny;
    l.nxt = nx + 2 * l.dn;
    const int r0 = (l.nxt - 1) % TILE;
    l.off = 0;
    if (r0 < l.dn - 1) l.off = ((l.dn - 1 - r0) + 3) / 4 * 4;
    l.ntiles = (l.off + l.nxt + TILE - 1) / TILE;
    l.pitch = l.ntiles * TILE;
    // side strips: each holds its dn CPML columns and at most 32*kstrip
    // columns; in narrow grids they share the interior columns between them
    l.kstrip = (l.dn + 31) / 32;
    const int sw = 32 * l.kstrip;
    l.sl = std::min(sw, l.dn + nx / 2);
    l.sr = std::max(l.nxt - sw, l.sl);
    return l;
}

// Snapshot events of the reference's counter: l starts at 1, is incremented
// every step k = 2..nt and triggers (and resets) when it equals store_snap.
std::vector<int> snapshot_steps(int nt, int store_snap) {
    std::vector<int> ks;
    int l = 1;
    for (int k = 2; k <= nt; ++k) {
        l = l + 1;
        if (l == store_snap) {
            ks.push_back(k);
            l = 0;
        }
    }
    return ks;
}

// Injection cells of one shot: interior cells only (the source array only
// enters the interior update), last writer wins for repeated cells
// (solver_acoustic_SS.f90:320-329).
std::vector<SrcEnt> injection_cells(const std::vector<int>& xs, const std::vector<int>& ys, const Layout& l) {
    std::map<std::pair<int, int>, int> last;
    for (size_t j = 0; j < xs.size(); ++j) {
        const int pr = l.dn + ys[j] - 1, pc = l.dn + xs[j] - 1;
        if (pr < l.dn || pr >= l.dn + l.ny || pc < l.dn || pc >= l.dn + l.nx) continue;
        last[{pr, pc}] = (int)j;
    }
    std::vector<SrcEnt> out;
    for (auto& kv : last) out.push_back(SrcEnt{kv.first.first, l.off + kv.first.second, kv.second});
    return out;
}

// One work item; its sources and receivers are the cells of physical
// columns [c0, c1) in rows [y0, y1).
static void append_item(Lists& L_, std::vector<WorkItem>& items, std::vector<SrcEnt>& srcs, const std::vector<SrcEnt>& cells,
                 const std::vector<RecEnt>& recs_shot, int shot, int tile, int y0, int y1, int kind, bool with_recs,
                 int c0, int c1) {
    WorkItem it{};
    it.shot = shot;
    it.tile = tile;
    it.y0 = y0;
    it.y1 = y1;
    it.kind = kind;
    std::vector<SrcEnt> sel;
    for (auto& c : cells)
        if (c.row >= y0 && c.row < y1 && c.col >= c0 && c.col < c1) sel.push_back(c);
    std::stable_sort(sel.begin(), sel.end(), [](const SrcEnt& a, const SrcEnt& b) { return a.row < b.row; });
    it.s0 = (int)srcs.size();
    srcs.insert(srcs.end(), sel.begin(), sel.end());
    it.s1 = (int)srcs.size();
    it.r0 = it.r1 = (int)L_.recs.size();
    if (with_recs) {
        std::vector<RecEnt> rs;
        for (auto& r : recs_shot)
            if (r.row >= y0 && r.row < y1 && r.col >= c0 && r.col < c1) rs.push_back(r);
        std::stable_sort(rs.begin(), rs.end(), [](const RecEnt& a, const RecEnt& b) { return a.row < b.row; });
        L_.recs.insert(L_.recs.end(), rs.begin(), rs.end());
        it.r1 = (int)L_.recs.size();
    }
    items.push_back(it);
}

// One two-step tile: output columns [x0, x0 + 120) (stored within [c0, c1))
// of rows [y0, y1); its sources are the cells of its whole first-step region,
// rows [y0 - R, y1 + R) and columns [x0 - 4, x0 + 124); its receivers the
// cells it stores.
static void append_two_step(Lists& L_, std::vector<WorkItem>& items, std::vector<SrcEnt>& srcs,
                     const std::vector<SrcEnt>& cells, const std::vector<RecEnt>& recs_shot, int shot, int x0, int y0,
                     int y1, int R, bool with_recs, int c0, int c1) {
    WorkItem it{};
    it.shot = shot;
    it.tile = x0;
    it.y0 = y0;
    it.y1 = y1;
    it.kind = 4;
    std::vector<SrcEnt> sel;
    for (auto& c : cells)
        if (c.row >= y0 - R && c.row < y1 + R && c.col >= x0 - 4 && c.col < x0 + 124) sel.push_back(c);
    std::stable_sort(sel.begin(), sel.end(), [](const SrcEnt& a, const SrcEnt& b) { return a.row < b.row; });
    it.s0 = (int)srcs.size();
    srcs.insert(srcs.end(), sel.begin(), sel.end());
    it.s1 = (int)srcs.size();
    it.r0 = it.r1 = (int)L_.recs.size();
    if (with_recs) {
        std::vector<RecEnt> rs;
        for (auto& r : recs_shot)
            if (r.row >= y0 && r.row < y1 && r.col >= std::max(c0, x0) && r.col < std::min(c1, x0 + 120))
                rs.push_back(r);
        std::stable_sort(rs.begin(), rs.end(), [](const RecEnt& a, const RecEnt& b) { return a.row < b.row; });
        L_.recs.insert(L_.recs.end(), rs.begin(), rs.end());
        it.r1 = (int)L_.recs.size();
    }
    items.push_back(it);
}

// A shot gets two-step tiles when the first-step cells around its interior
// columns are plain interior cells: R model columns on either side of
// [sl, sr) (no CPML column, no clamp) and at least one model row above the
// last R (which border the bottom pad and stay single-step).
bool two_step_ok(const Layout& l) {
    const int R = l.acc;
    return l.sl < l.sr && l.sl - R >= l.dn && l.sr + R <= l.dn + l.nx && l.ny > R;
}

// Work lists for a set of shots (local shot index = position in `geoms`).
// All shots share dn (one acc / dpml per launch), hence one kstrip.
// fband > 0 also builds the two-step lists (two-step tiles in bands of fband
// rows); eband > 0 gives the edge tiles their own height (see below).
Lists build_lists(const std::vector<ShotGeom>& geoms, const std::vector<Layout>& lays, int band_rows, int fband,
                  int eband) {
    Lists out;
    std::vector<WorkItem> sbot_f, sbot_a, strip_f, strip_a, bot_f, bot_a;
    // interior items grouped [shot][band] (a band = the tiles of one row band)
    std::vector<std::vector<std::vector<WorkItem>>> main_f, main_a, fus_f, fus_a, edge_f, edge_a;
    if (!lays.empty()) out.kstrip = lays[0].kstrip;
    auto bands = [](int n, int rows, auto&& fn) {
        const int nb = std::max(1, (n + rows - 1) / rows);
        for (int b = 0; b < nb; ++b) {
            const int y0 = (int)((long long)n * b / nb), y1 = (int)((long long)n * (b + 1) / nb);
            if (y1 > y0) fn(y0, y1);
        }
    };
    for (size_t s = 0; s < geoms.size(); ++s) {
        const Layout& l = lays[s];
        const ShotGeom& g = geoms[s];
        const auto cells_f = injection_cells(g.nxS, g.nyS, l);
        const auto cells_a = injection_cells(g.nxR, g.nyR, l);
        std::vector<RecEnt> recs;
        for (size_t i = 0; i < g.nxR.size(); ++i) {
            const int pr = l.dn + g.nyR[i] - 1, pc = l.dn + g.nxR[i] - 1;
            if (pr < l.dn) continue;  // top pad: identically zero, never recorded
            recs.push_back(RecEnt{pr, l.off + pc, (int)i});
        }
        std::vector<SrcEnt> none;
        const int xa = l.off + l.sl, xb = l.off + l.sr;  // interior columns, physical
        const int yb0 = l.nyt - l.dn;                    // first bottom pad row
        // interior columns: 128-column tiles, model rows in bands of band_rows,
        // bottom pad rows in bands of about BOTTOM_BAND (the y-phi is
        // ping-ponged, so bands are independent)
        if (xa < xb) {
            auto interior = [&](std::vector<std::vector<WorkItem>>& gf, std::vector<std::vector<WorkItem>>& ga,
                                int y0, int y1) {
                std::vector<WorkItem> vf, va;
                for (int t = xa / TILE; t <= (xb - 1) / TILE; ++t) {
                    const int c0 = std::max(t * TILE, xa), c1 = std::min((t + 1) * TILE, xb);
                    append_item(out, vf, out.src_fwd, cells_f, recs, (int)s, t, l.dn + y0, l.dn + y1, 0, true, c0,
                                c1);
                    append_item(out, va, out.src_adj, cells_a, recs, (int)s, t, l.dn + y0, l.dn + y1, 0, false, c0,
                                c1);
                }
                gf.push_back(vf);
                ga.push_back(va);
            };
            main_f.emplace_back();
            main_a.emplace_back();
            bands(l.ny, band_rows, [&](int y0, int y1) { interior(main_f.back(), main_a.back(), y0, y1); });
            if (fband > 0) {
                if (two_step_ok(l)) {
                    // model rows but the last R in two-step tiles of 120 columns; the last R rows
                    // as single-step tiles
                    const int R = l.acc, nr = l.ny - R;
                    fus_f.emplace_back();
                    fus_a.emplace_back();
                    edge_f.emplace_back();
                    edge_a.emplace_back();
                    // core: the wavefield cells a tile reads, rows [y0-2R-1, y1+2R] and columns
                    // [x0-8, x0+128), are two-step cells or the top pad; the other tiles are edge
                    // tiles (next to the side strips or the rows next to the bottom pad), which run
                    // beside the single-step lists on the pass's critical path
                    auto is_core = [&](int x0, int y1) {
                        return x0 - 8 >= xa && x0 + 128 <= xb && l.dn + y1 + 2 * R < l.dn + nr;
                    };
                    auto tile = [&](std::vector<WorkItem>& vf, std::vector<WorkItem>& va, int x0, int y0, int y1) {
                        append_two_step(out, vf, out.src_fwd, cells_f, recs, (int)s, x0, l.dn + y0, l.dn + y1, R,
                                        true, xa, xb);
                        out.fus_cells += (double)(y1 - y0) * (std::min(x0 + 120, xb) - std::max(x0, xa));
                        append_two_step(out, va, out.src_adj, cells_a, recs, (int)s, x0, l.dn + y0, l.dn + y1, R,
                                        false, xa, xb);
                    };
                    const int eb = std::min(nr, std::max(eband, 2 * R + 1));
                    if (eband <= 0 || nr - eb < 1) {
                        // one band height for all tiles
                        bands(nr, fband, [&](int y0, int y1) {
                            std::vector<WorkItem> vf, va, ef, ea;
                            for (int x0 = xa & ~3; x0 < xb; x0 += 120) {
                                const bool core = is_core(x0, y1);
                                tile(core ? vf : ef, core ? va : ea, x0, y0, y1);
                            }
                            fus_f.back().push_back(vf);
                            fus_a.back().push_back(va);
                            edge_f.back().push_back(ef);
                            edge_a.back().push_back(ea);
                        });
                    } else {
                        // a bottom edge band of eb rows: the rows [0, nr-eb) in bands of fband rows
                        // (core tiles, and edge tiles in the side tile columns), then the last eb
                        // rows -- the tiles whose second step reaches the single-step rows -- as one
                        // band of edge tiles, so that most of the model rows' bottom band is core
                        const int nc = nr - eb;
                        bands(nc, fband, [&](int y0, int y1) {
                            std::vector<WorkItem> vf, va, ef, ea;
                            for (int x0 = xa & ~3; x0 < xb; x0 += 120) {
                                const bool core = is_core(x0, y1);
                                tile(core ? vf : ef, core ? va : ea, x0, y0, y1);
                            }
                            fus_f.back().push_back(vf);
                            fus_a.back().push_back(va);
                            edge_f.back().push_back(ef);
                            edge_a.back().push_back(ea);
                        });
                        std::vector<WorkItem> ef, ea;
                        for (int x0 = xa & ~3; x0 < xb; x0 += 120) tile(ef, ea, x0, nc, nr);
                        edge_f.back().push_back(ef);
                        edge_a.back().push_back(ea);
                    }
                    for (int t = xa / TILE; t <= (xb - 1) / TILE; ++t) {
                        const int c0 = std::max(t * TILE, xa), c1 = std::min((t + 1) * TILE, xb);
                        append_item(out, out.lft_fwd, out.src_fwd, cells_f, recs, (int)s, t, l.dn + nr, l.dn + l.ny,
                                    0, true, c0, c1);
                        append_item(out, out.lft_adj, out.src_adj, cells_a, recs, (int)s, t, l.dn + nr, l.dn + l.ny,
                                    0, false, c0, c1);
                    }
                } else {
                    for (auto& b : main_f.back()) out.lft_fwd.insert(out.lft_fwd.end(), b.begin(), b.end());
                    for (auto& b : main_a.back()) out.lft_adj.insert(out.lft_adj.end(), b.begin(), b.end());
                }
            }
            bands(l.dn, std::min(BOTTOM_BAND, band_rows), [&](int j0, int j1) {
                for (int t = xa / TILE; t <= (xb - 1) / TILE; ++t) {
                    const int c0 = std::max(t * TILE, xa), c1 = std::min((t + 1) * TILE, xb);
                    append_item(out, bot_f, out.src_fwd, none, recs, (int)s, t, yb0 + j0, yb0 + j1, 1, true, c0, c1);
                    append_item(out, bot_a, out.src_adj, none, recs, (int)s, t, yb0 + j0, yb0 + j1, 1, false, c0, c1);
                }
            });
        }
        // side strips: model rows and bottom pad rows
        for (int side = 0; side < 2; ++side) {
            const int c0 = l.off + (side ? l.sr : 0), c1 = l.off + (side ? l.nxt : l.sl);
            if (c1 <= c0) continue;
            // model-row strips in bands of STRIP_BAND rows, or of the interior
            // items' height when that is shorter (a small grid: more warps,
            // shorter row marches; the bottom pad's bands follow it too)
            bands(l.ny, std::min(STRIP_BAND, band_rows), [&](int y0, int y1) {
                append_item(out, strip_f, out.src_fwd, cells_f, recs, (int)s, side, l.dn + y0, l.dn + y1, 2, true,
                            c0, c1);
                append_item(out, strip_a, out.src_adj, cells_a, recs, (int)s, side, l.dn + y0, l.dn + y1, 2, false,
                            c0, c1);
            });
            bands(l.dn, std::min(STRIP_BOTTOM_BAND, band_rows), [&](int j0, int j1) {
                append_item(out, sbot_f, out.src_fwd, none, recs, (int)s, side, yb0 + j0, yb0 + j1, 3, true, c0, c1);
                append_item(out, sbot_a, out.src_adj, none, recs, (int)s, side, yb0 + j0, yb0 + j1, 3, false, c0,
                            c1);
            });
        }
    }
    // Interior list: band after band across the shots.  Shot after shot keeps
    // the warps resident at any moment on a few shots' buffers, and the step
    // runs 13 % slower (measured on the 64-shot, 400 x 2000 workload).
    auto flatten = [](std::vector<std::vector<std::vector<WorkItem>>>& g, std::vector<WorkItem>& dst) {
        size_t nb = 0;
        for (auto& sh : g) nb = std::max(nb, sh.size());
        for (size_t b = 0; b < nb; ++b)
            for (auto& sh : g)
                if (b < sh.size()) dst.insert(dst.end(), sh[b].begin(), sh[b].end());
    };
    flatten(main_f, out.int_fwd);
    flatten(main_a, out.int_adj);
    flatten(fus_f, out.fus_fwd);
    flatten(fus_a, out.fus_adj);
    out.ncore = (int)out.fus_fwd.size();
    flatten(edge_f, out.fus_fwd);
    flatten(edge_a, out.fus_adj);
    // boundary lists: the strip warps (the short bottom-row bands first), then the bottom tiles
    out.nstrip = (int)(sbot_f.size() + strip_f.size());
    for (auto* v : {&sbot_f, &strip_f, &bot_f}) out.bnd_fwd.insert(out.bnd_fwd.end(), v->begin(), v->end());
    for (auto* v : {&sbot_a, &strip_a, &bot_a}) out.bnd_adj.insert(out.bnd_adj.end(), v->begin(), v->end());
    return out;
}

std::vector<StepUnit> plan_steps(int k0, int k1, const std::vector<int>& sn, bool two_step, bool snap_ok) {
    std::vector<StepUnit> units;
    int npass = 0;
    for (int k = k0; k <= k1;) {
        const int s0 = sn[k];
        if (two_step && k + 1 <= k1 && sn[k + 1] < 0 && (s0 < 0 || snap_ok)) {
            units.push_back({k, s0, true});
            ++npass;
            k += 2;
        } else {
            units.push_back({k, s0, false});
            k += 1;
        }
    }
    if (npass & 1) {  // the last pass becomes two single steps
        for (size_t i = units.size(); i-- > 0;)
            if (units[i].pass) {
                const StepUnit u = units[i];
                units[i] = {u.k, u.sn, false};
                units.insert(units.begin() + i + 1, StepUnit{u.k + 1, -1, false});
                break;
            }
    }
    return units;
}

}  // namespace fwi
