// Grid layout and work lists of the FWI time-step kernels: host-only code
// (no CUDA dependency), shared by the library and the CPU checks of the
// lists (tests/test_work_lists.py).
#pragma once
#include <vector>

#include "fwi_items.h"

namespace fwi {

struct Layout {
    int ny, nx, dn, nyt, nxt, off, pitch, ntiles;
    int sl, sr;   // side strips [0, sl) and [sr, nxt), interior columns [sl, sr)
    int kstrip;   // columns per lane of a strip warp: strips are at most 32*kstrip wide
    int acc;      // stencil half-width R
};

Layout make_layout(int ny, int nx, int acc, int dpml);

// Snapshot events of the reference's counter: l starts at 1, is incremented
// every step k = 2..nt and triggers (and resets) when it equals store_snap.
std::vector<int> snapshot_steps(int nt, int store_snap);

struct ShotGeom {
    int x0 = 0, nx = 0;
    std::vector<int> nxS, nyS, nxR, nyR;  // 1-based, window-relative
};

// Work items of one time step: interior items (128-column tiles of the model
// rows) for k_step_interior, boundary items (side strips for k_step_strip,
// then bottom-pad tiles for k_step_bottom), and the two-step lists; forward
// lists inject the sources and record the receivers, adjoint lists inject the
// adjoint sources at the receivers.
struct Lists {
    // boundary lists: nstrip side-strip items (bottom rows first), then the bottom tiles
    std::vector<WorkItem> int_fwd, int_adj, bnd_fwd, bnd_adj;
    // two-step passes: two-step tiles (kind 4; the first ncore of them core tiles, which read
    // no cell of the single-step lists) and the interior items outside them (kind 0)
    std::vector<WorkItem> fus_fwd, fus_adj, lft_fwd, lft_adj;
    int ncore = 0;
    double fus_cells = 0.0;  // cells the two-step tiles store (per step)
    int nstrip = 0, kstrip = 1;
    std::vector<SrcEnt> src_fwd, src_adj;
    std::vector<RecEnt> recs;
};

constexpr int TWO_STEP_BAND = 64;     // rows per two-step tile
constexpr int BOTTOM_BAND = 9;        // rows per bottom-tile work item
constexpr int STRIP_BAND = 16;        // rows per side-strip work item (model rows)
constexpr int STRIP_BOTTOM_BAND = 5;  // rows per side-strip work item (bottom pad rows)

// Injection cells of one shot (interior cells only, last writer wins).
std::vector<SrcEnt> injection_cells(const std::vector<int>& xs, const std::vector<int>& ys, const Layout& l);

// Whether a shot's interior can run as two-step tiles.
bool two_step_ok(const Layout& l);

// Work lists for a set of shots (local shot index = position in `geoms`);
// fband > 0 also builds the two-step lists (two-step tiles in bands of fband
// rows); eband > 0 makes the last max(eband, 2R+1) two-step rows -- the rows
// whose second step reaches the single-step rows next to the bottom pad --
// one band of edge tiles, the rows above it bands of fband rows (edge tiles
// only in the tile columns next to the side strips).
Lists build_lists(const std::vector<ShotGeom>& geoms, const std::vector<Layout>& lays, int band_rows, int fband = 0,
                  int eband = 0);

// One unit of a time loop: a two-step pass (steps k, k+1) or a single step
// k; sn = the snapshot block step k stores or images with, -1 for none.
struct StepUnit {
    int k, sn;
    bool pass;
};

// Steps k0..k1 (sn[k]: snapshot block of step k or -1; sn.size() > k1) as
// two-step passes and single steps: a pair (k, k+1) is a pass when
// two_step, step k+1 has no snapshot and step k has none or snap_ok; the
// number of passes is even (the last one becomes two single steps when it
// is not), so the state returns to the buffer pair it started in.
std::vector<StepUnit> plan_steps(int k0, int k1, const std::vector<int>& sn, bool two_step, bool snap_ok);

}  // namespace fwi
