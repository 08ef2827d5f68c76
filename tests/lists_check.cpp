// CPU checks of the step kernels' work lists (fwi_lists.cpp), over many grid
// shapes:
//  * single-step lists: every cell of the model rows and the bottom pad rows
//    (all columns) is updated by exactly one item;
//  * two-step passes: every interior cell of the model rows is stored by
//    exactly one two-step tile or leftover item, and nothing else;
//  * a two-step tile's first-step cells that its second step uses are plain
//    interior cells (no CPML column, no bottom pad row), its reads stay inside
//    the field, and core tiles read no cell a single-step item writes;
//  * source and receiver lists are sorted by row and lie inside the item;
//  * the time-loop planner (two-step passes and single steps) keeps its
//    invariants on random loops;
//  * the two-step pipeline is race-free: over three passes, kernels the
//    stream order and events leave unordered never write a wavefield cell
//    another one reads or writes (and dropping any one dependency edge
//    produces such a conflict).
// Prints "all ok" and exits 0, or prints the first failure and exits 1.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "fwi_lists.h"

using namespace fwi;

namespace {

unsigned rng_state = 12345u;
int rnd(int n) {
    rng_state = rng_state * 1664525u + 1013904223u;
    return (int)((rng_state >> 8) % (unsigned)n);
}

int fails = 0;
#define CHECK(cond, ...)                   \
    do {                                   \
        if (!(cond)) {                     \
            std::printf(__VA_ARGS__);      \
            std::printf("\n");             \
            ++fails;                       \
            return;                        \
        }                                  \
    } while (0)

// columns [c0, c1) of a single-step item
void item_cols(const WorkItem& it, const Layout& l, int& c0, int& c1) {
    const int xa = l.off + l.sl, xb = l.off + l.sr;
    if (it.kind == 0 || it.kind == 1) {
        c0 = std::max(it.tile * TILE, xa);
        c1 = std::min((it.tile + 1) * TILE, xb);
    } else {
        c0 = l.off + (it.tile ? l.sr : 0);
        c1 = l.off + (it.tile ? l.nxt : l.sl);
    }
}

void check(int ny, int nx, int acc, int dpml, int nsrc, int band, int fband, int eband = 0) {
    const Layout l = make_layout(ny, nx, acc, dpml);
    ShotGeom g;
    g.nx = nx;
    for (int i = 0; i < nsrc; ++i) {
        g.nxS.push_back(1 + rnd(nx));
        g.nyS.push_back(1 + rnd(ny));
    }
    for (int i = 0; i < 60; ++i) {
        g.nxR.push_back(1 + rnd(nx));
        g.nyR.push_back(1 + rnd(ny));
    }
    const Lists L = build_lists({g}, {l}, band, fband, eband);
    const int R = l.acc, xa = l.off + l.sl, xb = l.off + l.sr;
    const size_t n = (size_t)l.nyt * l.pitch;
    auto at = [&](int y, int c) { return (size_t)y * l.pitch + c; };

    // single-step lists: model rows and bottom pad rows, columns [0, nxt)
    std::vector<int> own(n, 0);
    for (const auto* v : {&L.int_fwd, &L.bnd_fwd})
        for (const WorkItem& it : *v) {
            int c0, c1;
            item_cols(it, l, c0, c1);
            for (int y = it.y0; y < it.y1; ++y)
                for (int c = c0; c < c1; ++c) own[at(y, c)]++;
            for (int i = it.s0; i < it.s1; ++i) {
                const SrcEnt& e = L.src_fwd[i];
                CHECK(e.row >= it.y0 && e.row < it.y1 && e.col >= c0 && e.col < c1, "single-step source outside its item");
                CHECK(i == it.s0 || L.src_fwd[i - 1].row <= e.row, "single-step sources not sorted");
            }
        }
    for (int y = 0; y < l.nyt; ++y)
        for (int c = 0; c < l.pitch; ++c) {
            const bool upd = y >= l.dn && c >= l.off && c < l.off + l.nxt;
            CHECK(own[at(y, c)] == (upd ? 1 : 0), "single step: cell (%d,%d) updated %d times (ny %d nx %d acc %d dpml %d)",
                  y, c, own[at(y, c)], ny, nx, acc, dpml);
        }
    if (fband <= 0) return;

    // two-step lists
    std::fill(own.begin(), own.end(), 0);
    const int ylast = l.nyt - l.dn - R;  // first leftover row
    for (size_t k = 0; k < L.fus_fwd.size(); ++k) {
        const WorkItem& it = L.fus_fwd[k];
        const int x0 = it.tile;
        CHECK(it.kind == 4 && x0 % 4 == 0, "two-step tile misaligned");
        CHECK(it.y0 >= l.dn && it.y1 <= ylast, "two-step tile rows outside [dn, nyt-dn-R)");
        // reads: p_n rows [y0-2R-1, y1+2R], columns [x0-8, x0+128)
        const long long lo = (long long)(it.y0 - 2 * R - 1) * l.pitch + x0 - 8;
        const long long hi = (long long)(it.y1 + 2 * R) * l.pitch + x0 + 128;
        CHECK(lo >= 0 && hi <= (long long)n, "two-step tile reads outside the field");
        // first-step cells used by the second step are plain interior cells
        const int ca = std::max(x0, xa) - R, cb = std::min(x0 + 120, xb) + R;
        CHECK(ca >= l.off + l.dn && cb <= l.off + l.dn + l.nx, "two-step halo columns not plain");
        CHECK(it.y1 + R <= l.nyt - l.dn, "two-step halo rows reach the bottom pad");
        for (int y = it.y0; y < it.y1; ++y)
            for (int c = std::max(x0, xa); c < std::min(x0 + 120, xb); ++c) own[at(y, c)]++;
        if ((int)k < L.ncore)
            for (int y = it.y0 - 2 * R - 1; y <= it.y1 + 2 * R; ++y)
                for (int c = x0 - 8; c < x0 + 128; ++c) {
                    const bool top = y < l.dn, two = y < ylast && c >= xa && c < xb;
                    CHECK(top || two, "core tile reads single-step cell (%d,%d)", y, c);
                }
        for (int i = it.s0; i < it.s1; ++i) {
            const SrcEnt& e = L.src_fwd[i];
            CHECK(e.row >= it.y0 - R && e.row < it.y1 + R && e.col >= x0 - 4 && e.col < x0 + 124,
                  "two-step source outside the first-step region");
            CHECK(i == it.s0 || L.src_fwd[i - 1].row <= e.row, "two-step sources not sorted");
        }
        for (int i = it.r0; i < it.r1; ++i) {
            const RecEnt& r = L.recs[i];
            CHECK(r.row >= it.y0 && r.row < it.y1 && r.col >= std::max(x0, xa) && r.col < std::min(x0 + 120, xb),
                  "two-step receiver outside the stored cells");
            CHECK(i == it.r0 || L.recs[i - 1].row <= r.row, "two-step receivers not sorted");
        }
    }
    for (const WorkItem& it : L.lft_fwd) {
        int c0, c1;
        item_cols(it, l, c0, c1);
        for (int y = it.y0; y < it.y1; ++y)
            for (int c = c0; c < c1; ++c) own[at(y, c)]++;
    }
    if (xa < xb)
        for (int y = 0; y < l.nyt; ++y)
            for (int c = 0; c < l.pitch; ++c) {
                const bool in = y >= l.dn && y < l.dn + ny && c >= xa && c < xb;
                CHECK(own[at(y, c)] == (in ? 1 : 0), "two-step: cell (%d,%d) stored %d times (two_step_ok %d)", y, c,
                      own[at(y, c)], (int)two_step_ok(l));
            }
    if (two_step_ok(l)) CHECK(!L.fus_fwd.empty(), "a two-step shot without tiles");
}

// The step planner: every step of k0..k1 once and in order, a pass never
// has a snapshot in its second step nor, unless allowed, in its first, the
// number of passes is even, and no pass is made when two-step is off.
void check_plan(int k0, int k1, const std::vector<int>& sn, bool two, bool snap_ok) {
    const std::vector<StepUnit> u = plan_steps(k0, k1, sn, two, snap_ok);
    int k = k0, npass = 0;
    for (const StepUnit& x : u) {
        CHECK(x.k == k, "plan: step %d expected, got %d", k, x.k);
        CHECK(x.sn == sn[x.k], "plan: wrong snapshot block at step %d", x.k);
        if (x.pass) {
            CHECK(two, "plan: pass without two-step");
            CHECK(x.k + 1 <= k1 && sn[x.k + 1] < 0, "plan: snapshot in the second step of a pass at %d", x.k);
            CHECK(snap_ok || x.sn < 0, "plan: snapshot in a pass at %d", x.k);
            ++npass;
            k += 2;
        } else {
            k += 1;
        }
    }
    CHECK(k == k1 + 1, "plan: steps %d..%d not all planned (%d)", k0, k1, k);
    CHECK(npass % 2 == 0, "plan: odd number of passes");
}

// The two-step pipeline (two_step_run in fwi_host.cu): the kernels of three
// consecutive passes with their wavefield read sets (the cells whose values
// are used) and write sets, per buffer of the two pairs; every two kernels
// that the pipeline's stream order and events leave unordered must not have
// one write what the other reads or writes.  The dependency edges below
// mirror two_step_run: C (core tiles, main stream), E (edge tiles, after A2
// on the second stream), A2/B2 (leftover interior rows and bottom tiles,
// second stream), A3/B3 (side strips, third stream).
struct Kern {
    const char* name;
    int pass;
    std::vector<std::vector<char>> rd, wr;  // [buffer 0..3][cell]
    std::vector<int> deps;                  // direct predecessors
};

void check_pipeline(int ny, int nx, int acc, int dpml, int fband, int eband = 0) {
    const Layout l = make_layout(ny, nx, acc, dpml);
    if (!two_step_ok(l)) return;
    ShotGeom g;
    g.nx = nx;
    const Lists L = build_lists({g}, {l}, 16, fband, eband);
    const int R = l.acc;
    const size_t n = (size_t)l.nyt * l.pitch;
    auto cur = [](int k, int pair) { return 2 * pair + ((k & 1) ? 0 : 1); };
    auto prev = [](int k, int pair) { return 2 * pair + ((k & 1) ? 1 : 0); };
    std::vector<Kern> K;
    auto mk = [&](const char* name, int pass) {
        Kern k{name, pass, std::vector<std::vector<char>>(4, std::vector<char>(n, 0)),
               std::vector<std::vector<char>>(4, std::vector<char>(n, 0)), {}};
        K.push_back(k);
        return (int)K.size() - 1;
    };
    auto box = [&](std::vector<char>& m, int ya, int yb, int ca, int cb) {  // rows [ya, yb), cols [ca, cb), clipped
        for (int y = std::max(ya, 0); y < std::min(yb, l.nyt); ++y)
            for (int c = std::max(ca, 0); c < std::min(cb, l.pitch); ++c) m[(size_t)y * l.pitch + c] = 1;
    };
    const int xa = l.off + l.sl, xb = l.off + l.sr;
    // single-step item at step k reading pair (rp, rp1) and writing wo
    auto single = [&](Kern& kk, const WorkItem& it, int rp, int rp1, int wo) {
        int c0, c1;
        item_cols(it, l, c0, c1);
        box(kk.wr[wo], it.y0, it.y1, c0, c1);
        box(kk.rd[rp], it.y0 - R, it.y1 + R, c0 - R, c1 + R);
        box(kk.rd[rp1], it.y0, it.y1, c0, c1);
    };
    auto tiles = [&](Kern& kk, int from, int to, int k, int X, int Y) {
        for (int i = from; i < to; ++i) {
            const WorkItem& it = L.fus_fwd[i];
            const int o0 = std::max(it.tile, xa), o1 = std::min(it.tile + 120, xb);
            box(kk.wr[prev(k, Y)], it.y0, it.y1, o0, o1);
            box(kk.wr[prev(k + 1, Y)], it.y0, it.y1, o0, o1);
            box(kk.rd[cur(k, X)], std::max(it.y0 - 2 * R, l.dn), it.y1 + 2 * R, o0 - 2 * R, o1 + 2 * R);
            box(kk.rd[prev(k, X)], std::max(it.y0 - R, l.dn), it.y1 + R, o0 - R, o1 + R);
        }
    };
    const int nstrip = L.nstrip, nb = (int)L.bnd_fwd.size();
    int lastC = -1, lastE = -1, lastA3 = -1, lastB2 = -1, lastB3 = -1, lastst2 = -1;
    for (int j = 0, k = 2, X = 0; j < 3; ++j, k += 2, X ^= 1) {
        const int Y = X ^ 1;
        const int c = mk("C", j), e = mk("E", j), a2 = mk("A2", j), a3 = mk("A3", j), b2 = mk("B2", j),
                  b3 = mk("B3", j);
        tiles(K[c], 0, L.ncore, k, X, Y);
        tiles(K[e], L.ncore, (int)L.fus_fwd.size(), k, X, Y);
        for (const WorkItem& it : L.lft_fwd) {
            single(K[a2], it, cur(k, X), prev(k, X), prev(k, Y));
            single(K[b2], it, cur(k + 1, Y), cur(k, X), prev(k + 1, Y));
        }
        for (int i = nstrip; i < nb; ++i) {
            single(K[a2], L.bnd_fwd[i], cur(k, X), prev(k, X), prev(k, Y));
            single(K[b2], L.bnd_fwd[i], cur(k + 1, Y), cur(k, X), prev(k + 1, Y));
        }
        for (int i = 0; i < nstrip; ++i) {
            single(K[a3], L.bnd_fwd[i], cur(k, X), prev(k, X), prev(k, Y));
            single(K[b3], L.bnd_fwd[i], cur(k + 1, Y), cur(k, X), prev(k + 1, Y));
        }
        auto dep = [&](int v, int u) {
            if (u >= 0) K[v].deps.push_back(u);
        };
        dep(c, lastC), dep(c, lastE);                      // C(j): stream order, E(j-1)
        dep(a3, lastA3 >= 0 ? lastB3 : -1), dep(a3, lastB2);  // A3(j): B3(j-1) (stream), B2(j-1)
        dep(a2, lastst2), dep(a2, lastB3);                 // A2(j): B2(j-1) (stream), B3(j-1)
        dep(e, a2), dep(e, lastC);                         // E(j): A2(j) (stream), C(j-1)
        dep(b3, a3), dep(b3, e);                           // B3(j): A3(j) (stream), E(j)
        dep(b2, e), dep(b2, a3);                           // B2(j): E(j) (stream), A3(j)
        lastC = c, lastE = e, lastA3 = a3, lastB2 = b2, lastB3 = b3, lastst2 = b2;
    }
    // reachability
    const int nk = (int)K.size();
    std::vector<std::vector<char>> reach(nk, std::vector<char>(nk, 0));
    for (bool grew = true; grew;) {  // transitive closure (edges do not follow creation order)
        grew = false;
        for (int v = 0; v < nk; ++v)
            for (int u : K[v].deps) {
                if (!reach[v][u]) reach[v][u] = 1, grew = true;
                for (int w = 0; w < nk; ++w)
                    if (reach[u][w] && !reach[v][w]) reach[v][w] = 1, grew = true;
            }
    }
    for (int a = 0; a < nk; ++a)
        for (int b = a + 1; b < nk; ++b) {
            if (reach[a][b] || reach[b][a]) continue;
            for (int buf = 0; buf < 4; ++buf)
                for (size_t i = 0; i < n; ++i) {
                    const bool ab = K[a].wr[buf][i] && (K[b].rd[buf][i] || K[b].wr[buf][i]);
                    const bool ba = K[b].wr[buf][i] && K[a].rd[buf][i];
                    CHECK(!ab && !ba, "pipeline race: %s(%d) and %s(%d) on buffer %d cell (%zu,%zu) (ny %d nx %d acc %d)",
                          K[a].name, K[a].pass, K[b].name, K[b].pass, buf, i / l.pitch, i % l.pitch, ny, nx, acc);
                }
        }
}

}  // namespace

int main() {
    for (int acc : {3, 4})
        for (int dpml : {8, 20})
            for (int nx : {90, 250, 400}) {
                check_pipeline(40 + nx % 37, nx, acc, dpml, 16 + nx % 20);
                check_pipeline(40 + nx % 37, nx, acc, dpml, 16 + nx % 20, 8 + nx % 9);
            }
    if (fails) return 1;
    for (int trial = 0; trial < 3000 && !fails; ++trial) {
        const int k0 = 2 + rnd(5), k1 = k0 - 1 + rnd(60);
        const int ss = 1 + rnd(12);
        std::vector<int> sn(k1 + 2, -1);
        for (int k = k0; k <= k1; ++k)
            if (k % ss == 0) sn[k] = k / ss;
        check_plan(k0, k1, sn, trial % 4 != 0, trial % 3 != 0);
    }
    check(400, 2000, 3, 20, 5, 16, 64);
    check(400, 2000, 3, 20, 5, 16, 48);
    check(400, 2000, 3, 20, 5, 16, 96);
    check(400, 2000, 4, 20, 5, 16, 64);
    check(600, 3000, 3, 20, 5, 16, 96);
    for (int eb : {1, 7, 8, 16, 32, 500}) {
        check(400, 2000, 3, 20, 5, 16, 64, eb);
        check(400, 2000, 4, 20, 5, 16, 48, eb);
    }
    check(37, 61, 3, 20, 3, 32, 48);
    check(12, 90, 4, 8, 3, 16, 64);
    for (int band : {1, 2, 3, 4, 5}) {  // short bands: the strips and the bottom pad follow them
        check(37, 61, 3, 20, 3, band, 48);
        check(200, 400, 4, 20, 2, band, 0);
        check(23, 150, 4, 8, 3, band, 16, 7);
    }
    int cases = 4;
    for (int nx = 20; nx < 400 && !fails; nx += 7)
        for (int dpml : {1, 5, 10, 20, 25, 30, 40, 54})
            for (int acc : {3, 4}) {
                if (dpml + 2 * acc > MAXDN - 2) continue;
                check(6 + nx % 53, nx, acc, dpml, 4, 8 + nx % 40, 16 + nx % 50);
                check(6 + nx % 53, nx, acc, dpml, 4, 8 + nx % 40, 16 + nx % 50, 4 + nx % 23);
                ++cases;
                if (fails) break;
            }
    if (fails) return 1;
    std::printf("all ok (%d grids)\n", cases);
    return 0;
}
