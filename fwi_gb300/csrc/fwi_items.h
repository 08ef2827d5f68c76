// Work items of the FWI time-step kernels: plain structs shared by the host
// work-list builder (fwi_lists.cpp, no CUDA dependency) and the kernels.
#pragma once

namespace fwi {

constexpr int TILE = 128;       // columns per warp tile (32 lanes x float4)
constexpr int MAXR = 4;         // largest supported FD half-order (acc)
constexpr int MAXDN = 64;       // largest supported CPML pad (dpml + 2*acc)

struct SrcEnt {                 // one injected source cell (deduplicated)
    int row;                    // padded row
    int col;                    // physical column
    int vidx;                   // index into the shot's value table [vidx][nt]
};
struct RecEnt {                 // one recorded receiver
    int row, col;               // padded row, physical column
    int ridx;                   // receiver index: Rec_point(:, ridx+1)
};

struct WorkItem {               // one warp's work in a step launch
    int shot;
    int tile;                   // tile index (x0 = tile*TILE physical); side strip: 0 left, 1 right;
                                // two-step tile: its first physical column
    int y0, y1;                 // padded rows [y0, y1)
    int kind;                   // 0 = interior model rows, 1 = bottom pad rows (interior columns),
                                // 2 = side strip, model rows; 3 = side strip, bottom pad rows;
                                // 4 = two-step interior tile
    int s0, s1;                 // SrcEnt range (sorted by row)
    int r0, r1;                 // RecEnt range (sorted by row)
    int pad_;
};

}  // namespace fwi
