// Internal device data structures of the FWI step kernels.
//
// Device layout of one shot (all fields float, row-major, x fastest):
//   rows 0..nyt-1 of the padded grid (nyt = dn + ny + dn, dn = dpml + 2*acc),
//   row pitch `pitch` floats (a multiple of TILE = 128), logical padded column
//   c stored at physical column off + c.  `off` (a multiple of 4) is chosen so
//   that the first 128-column tile holds the whole left CPML strip and the
//   last tile holds the whole right strip.
//   Model rows are split by column: the side strips [0, sl) and [sr, nxt)
//   (each at most 32*ceil(dn/32) columns wide, holding the x-CPML columns)
//   go to one warp per band with one column per lane; the interior columns
//   [sl, sr) go to 128-column tiles, one warp per tile and band (4 columns
//   per lane, float4), with stores masked to [sl, sr) in the two partial
//   tiles.  Bottom pad rows are split the same way (strip warps for the
//   corners and the columns next to them, 128-column tiles for [sl, sr)).
//   Every warp marches down its band with a register queue of 2*acc+1 rows.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "fwi_items.h"

namespace fwi {

struct ShotDev {
    float* pf[4];               // wavefield buffers: pair 0 (pf[0], pf[1]) and pair 1 (pf[2], pf[3]);
                                // StepParams::rp/rp1/wo/wo2 select them per launch
    const float* c2;            // c^2 dt^2 / d^2
    float* phx;                 // x-direction CPML phi (side strips and corners)
    float* chx;                 // x-direction chi
    float* phy;                 // y-direction phi (bottom strip and corners),
    float* phy2;                // ping-ponged with phy by step parity
    float* chy;                 // y-direction chi
    const float* srcv;          // injected values [vidx][nt]
    float* rec;                 // Rec_point(nt, nrec) column-major
    void* snaps;                // snapshots [s][ny][pitch] (float / 16-bit)
    float* sscale;              // 16-bit snapshot scales [s][ny][ntiles + 2] (tiles, then the two side strips)
    float* k32;                 // FP32 imaging accumulator [ny][pitch]
    double* k64;                // FP64 imaging accumulator [ny][pitch]
    long long snap_stride;      // elements per snapshot block (ny*pitch)
    int ny, nx, nyt, nxt;
    int off, pitch, ntiles, dn;
    int nt, nrec;
    int x0;                     // window start in the full model
    int sl, sr;                 // interior columns [sl, sr) (logical); side strips [0, sl), [sr, nxt)
    int pad_;
};

struct StepParams {
    const WorkItem* items;
    const ShotDev* shots;
    const SrcEnt* srcs;         // source cells of all items (sorted per item)
    const RecEnt* recs;         // receiver cells of all items (sorted per item)
    const float* fA;            // CPML factors (dn entries, 0-based)
    const float* fB;
    int nitems;
    int nstrip;                 // boundary list: the first nstrip items are side strips (kinds 2, 3),
                                // the bottom tiles follow
    int t;                      // k-2: source column / receiver row this step
    int parity;                 // k & 1: which y-phi buffer is current
    int rp, rp1, wo;            // wavefield buffers (ShotDev::pf): p, p_1 read; p_3 written (wo may be rp1)
    int wo2;                    // two-step tiles: buffer of the second step's p_3
    int snap;                   // snapshot block this step, -1 if none
    int snap_form;              // FWI_SNAP_*
    int grad_form;              // FWI_GRAD_*
    int record;                 // 1: record receivers
    float dt;                   // for ((p3-p1)*0.5)/dt
    float rdt;                  // RN(1/dt) for div_by_const (0: divide)
    float ss;                   // float(store_snap) for the imaging condition
    float c1[MAXR + 1];         // first-derivative taps
    float c2[MAXR + 1];         // second-derivative taps (centre halved)
};

}  // namespace fwi
