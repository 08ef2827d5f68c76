// FWI time-step kernels for sm_103a.
//
// Three launches advance every shot of a wave by one time step of the
// reference solver (solver_acoustic_SS.f90:313-586); a fourth,
// k_step2_interior, advances the interior of the model rows by two steps in
// one sweep (two-step passes, below):
//
//   k_step_interior  model rows dn..dn+ny-1, interior columns: interior
//                    update with source injection (:319-330, :433-434),
//                    snapshot store (:438-454) or imaging condition
//                    (:457-473), receiver recording (:551-555);
//   k_step_strip     model rows, the two side strips: left/right CPML strips
//                    (pml_matrices_x, solver_PML_matrices.f90:1-40) with the
//                    grid-edge clamps, and the interior columns next to them;
//   k_step_bottom    bottom pad rows: bottom CPML strip (pml_matrices_y
//                    :42-81) and the two bottom corners in two stages
//                    (pml_matrices_xycorner :83-112, solver_acoustic_SS.f90:395-411).
//
// The top pad rows are never written: with the free surface they stay
// exactly zero for the whole run (solver_acoustic_SS.f90:416-429, :477-479).
//
// Interior and bottom warps own a 128-column tile (4 columns per lane,
// float4) and march down a band of rows; the y-stencil comes from a register
// queue of 2R+1 rows, the x-stencil from warp shuffles of the current row
// plus one halo float4 at each end of the tile.  Strip warps hold one column
// per lane.  The wavefield lives in two buffer pairs (ShotDev::pf): a single
// step reads p and p_1 of one pair and writes p_3 over p_1 (each cell reads
// its own p_1 only); a two-step pass reads one pair and writes both new
// steps to the other.  Every cell is written by exactly one warp.  The CPML
// memory variables are updated in place: the strip-local derivative of phi
// only reads phi values of the same warp, loaded before they are overwritten.
//
// This file is compiled with --fmad=false: every a*b+c below is a rounded
// multiply followed by a rounded add, in the order the Fortran source writes
// the expression, so results are bit-identical to the reference arithmetic.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <climits>

#include "fwi_div.cuh"
#include "fwi_internal.cuh"

namespace fwi {

namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }

__device__ __forceinline__ void to_arr(float4 v, float* a) { a[0] = v.x; a[1] = v.y; a[2] = v.z; a[3] = v.w; }
__device__ __forceinline__ float4 from_arr(const float* a) { return make_float4(a[0], a[1], a[2], a[3]); }
// Packed FP32 pairs (Blackwell f32x2 add/fma: two independently rounded FP32
// operations per instruction), used by the interior and bottom updates.
// Products are formed as fma(a, b, +0): ptxas contracts a packed multiply
// feeding a packed add into a fused multiply-add (even with --fmad=false),
// which would change the rounding.  fma with a +0 addend is the correctly
// rounded product and is not contracted; it differs from a*b only in the
// sign of a zero product, which changes no nonzero value downstream (these
// updates only add and multiply).  An addend of -0 would keep the sign too,
// but then fma(a, b, -0) is a plain product to ptxas and is contracted
// again.  Lane columns (0,1) and (2,3) form the two pairs; x-neighbour pairs
// at odd offsets are re-paired.
__device__ __forceinline__ float2 pr(const float4& v, int k) { return k == 0 ? make_float2(v.x, v.y) : make_float2(v.z, v.w); }
__device__ __forceinline__ float2 mul0(float2 a, float2 b) { return __ffma2_rn(a, b, make_float2(0.f, 0.f)); }

__device__ __forceinline__ float sel(const float* a, int e) {
    return e == 0 ? a[0] : (e == 1 ? a[1] : (e == 2 ? a[2] : a[3]));
}
__device__ __forceinline__ float4 shfl_up4(float4 v) {
    return make_float4(__shfl_up_sync(FULL, v.x, 1), __shfl_up_sync(FULL, v.y, 1), __shfl_up_sync(FULL, v.z, 1),
                       __shfl_up_sync(FULL, v.w, 1));
}
__device__ __forceinline__ float4 shfl_dn4(float4 v) {
    return make_float4(__shfl_down_sync(FULL, v.x, 1), __shfl_down_sync(FULL, v.y, 1),
                       __shfl_down_sync(FULL, v.z, 1), __shfl_down_sync(FULL, v.w, 1));
}

// 12-value window of a row around this lane's 4 columns: w[4+e] is column e.
__device__ __forceinline__ void window(float4 c, float4 hl, float4 hr, int lane, float* w) {
    float4 l = shfl_up4(c), r = shfl_dn4(c);
    if (lane == 0) l = hl;
    if (lane == 31) r = hr;
    to_arr(l, w);
    to_arr(c, w + 4);
    to_arr(r, w + 8);
}

// space_deriv2y / space_derivy at the centre row of the queue (:38-45, :109-116)
template <int R>
__device__ __forceinline__ void yderivs(const float4* q, const StepParams& P, float* d2, float* d1) {
    float a[2 * R + 1][4];
#pragma unroll
    for (int i = 0; i <= 2 * R; ++i) to_arr(q[i], a[i]);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        float s2 = 0.f, s1 = 0.f;
#pragma unroll
        for (int i = 0; i <= R; ++i) {
            s2 = s2 + (a[R + i][e] + a[R - i][e]) * P.c2[i];
            s1 = s1 + (a[R + i][e] - a[R - i][e]) * P.c1[i];
        }
        d2[e] = s2;
        d1[e] = s1;
    }
}

// First derivative along y of the centre row of a queue (strip-local phi).
template <int R>
__device__ __forceinline__ void yderiv1(const float4* f, const StepParams& P, float* d1) {
    float a[2 * R + 1][4];
#pragma unroll
    for (int i = 0; i <= 2 * R; ++i) to_arr(f[i], a[i]);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        float s1 = 0.f;
#pragma unroll
        for (int i = 0; i <= R; ++i) s1 = s1 + (a[R + i][e] - a[R - i][e]) * P.c1[i];
        d1[e] = s1;
    }
}

// Snapshot store (forward) of the interior cells of one row:
// Fields(j, snap*nx+i) = (p_3 - p_1)*0.5/dt   (solver_acoustic_SS.f90:447)
// This lane stores elements [lo, hi) of its 4 columns; `seg` is the row
// segment whose scale the 16-bit forms use.
__device__ __forceinline__ void store_snapshot(const StepParams& P, const ShotDev& S, int yrow, int lane, int xl,
                                               int lo, int hi, const float* p3, const float* pm1, int seg) {
    float v[4];
    bool in[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        in[e] = (e >= lo) && (e < hi);
        v[e] = in[e] ? div_by_const((p3[e] - pm1[e]) * 0.5f, P.dt, P.rdt) : 0.f;
    }
    const bool full = in[0] && in[3];
    const size_t base = (size_t)P.snap * (size_t)S.snap_stride + (size_t)yrow * S.pitch + xl;
    if (P.snap_form == 0) {
        float* F = reinterpret_cast<float*>(S.snaps) + base;
        if (full) {
            st4(F, from_arr(v));
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (in[e]) F[e] = v[e];
        }
        return;
    }
    // 16-bit forms: power-of-two scale per row segment so that the largest
    // magnitude maps below 2^14 (exact scaling, no extra rounding).
    float m = fmaxf(fmaxf(fabsf(v[0]), fabsf(v[1])), fmaxf(fabsf(v[2]), fabsf(v[3])));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(FULL, m, o));
    int ex = 0;
    if (m > 0.f) frexpf(m, &ex);
    const int sh = 14 - ex;
    unsigned short h[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const float sv = ldexpf(v[e], sh);
        if (P.snap_form == 1) {
            __nv_bfloat16 b = __float2bfloat16_rn(sv);
            h[e] = *reinterpret_cast<unsigned short*>(&b);
        } else {
            __half b = __float2half_rn(sv);
            h[e] = *reinterpret_cast<unsigned short*>(&b);
        }
    }
    unsigned short* F = reinterpret_cast<unsigned short*>(S.snaps) + base;
    if (full) {
        uint2 pk;
        pk.x = (unsigned)h[0] | ((unsigned)h[1] << 16);
        pk.y = (unsigned)h[2] | ((unsigned)h[3] << 16);
        *reinterpret_cast<uint2*>(F) = pk;
    } else {
#pragma unroll
        for (int e = 0; e < 4; ++e)
            if (in[e]) F[e] = h[e];
    }
    if (lane == 0) S.sscale[((size_t)P.snap * S.ny + yrow) * (S.ntiles + 2) + seg] = ldexpf(1.f, -sh);
}

// Receiver recording for the row just finished (:553): every receiver in
// this cell gets p_3.
__device__ __forceinline__ void record_row(const StepParams& P, const ShotDev& S, int y, int xl, int& ri, int r1,
                                           int& rrow, const float* p3) {
    while (rrow == y) {
        const RecEnt r = P.recs[ri];
        if ((r.col >> 2) == (xl >> 2)) S.rec[(size_t)r.ridx * S.nt + P.t] = sel(p3, r.col & 3);
        ++ri;
        rrow = (ri < r1) ? P.recs[ri].row : INT_MAX;
    }
}

// Injected values of row y for the warp's 128 columns starting at physical
// column c0 (entries sorted by row, one per cell, all inside those columns;
// the cursor si at the first entry of row y).  The lanes take the row's
// entries 32 at a time and scatter their values into the warp's line `inj`
// (a float4 per lane, entry [1 + lane] for lane l's columns c0 + 4l ..);
// each lane then reads its own float4.  Called by the whole warp when srow == y.
__device__ __forceinline__ float4 gather_sources(const StepParams& P, const ShotDev& S, int y, int c0, int t, int& si,
                                                 int s1, int& srow, float4* inj, int lane) {
    inj[1 + lane] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncwarp();
    while (srow == y) {
        const int i = si + lane;
        bool mine = false;
        if (i < s1) {
            const SrcEnt e = P.srcs[i];
            mine = e.row == y;
            if (mine) reinterpret_cast<float*>(inj + 1)[e.col - c0] = __ldg(S.srcv + (size_t)e.vidx * S.nt + t);
        }
        si += __popc(__ballot_sync(FULL, mine));  // the row's entries are consecutive
        srow = (si < s1) ? P.srcs[si].row : INT_MAX;
    }
    __syncwarp();
    return inj[1 + lane];
}

// Receivers of row y (entries sorted by row, the cursor ri at the first one
// of row y): p_3 of the warp's 128 columns starting at physical column c0 is
// in `line` (entry [1 + lane] for lane l's columns c0 + 4l ..), visible to
// the whole warp; the lanes take the row's receivers 32 at a time.  Called by
// the whole warp when rrow == y.
__device__ __forceinline__ void record_row_par(const StepParams& P, const ShotDev& S, int y, int c0, int t, int& ri,
                                               int r1, int& rrow, const float4* line, int lane) {
    while (rrow == y) {
        const int i = ri + lane;
        bool mine = false;
        if (i < r1) {
            const RecEnt r = P.recs[i];
            mine = r.row == y;
            if (mine) S.rec[(size_t)r.ridx * S.nt + t] = reinterpret_cast<const float*>(line + 1)[r.col - c0];
        }
        ri += __popc(__ballot_sync(FULL, mine));  // the row's entries are consecutive
        rrow = (ri < r1) ? P.recs[ri].row : INT_MAX;
    }
}

}  // namespace

// Per-lane asynchronous prefetch of the rows a warp will need (cp.async,
// 16 bytes per lane per array, L2-only).  Every lane reads back only what it
// copied itself, so no intra-warp synchronisation is needed.
__device__ __forceinline__ void cp16(void* smem_dst, const void* gmem_src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// One prefetch stage of the bottom kernel: p(y+R), p_1(y), c2(y), y-phi(y),
// y-chi(y), the y-phi row the derivative queue needs next (jl+1+R), and the
// halo float4 of p(y).
constexpr int SB_P = 0, SB_P1 = 32, SB_C2 = 64, SB_PY = 96, SB_CY = 128, SB_FA = 160, SB_HL = 192, SB_HR = 193,
              SB_SIZE = 194;
constexpr int BOT_DEPTH = 3;
constexpr int BOT_SMEM = 4 * BOT_DEPTH * SB_SIZE * 16;

// Bottom pad rows [it.y0, it.y1) of one tile, interior columns [sl, sr)
// only: the bottom CPML strip (pml_matrices_y, solver_PML_matrices.f90:42-81);
// the corners lie in the side strips.  The first and last tile of the range
// may be partial: lanes outside it compute but store nothing.  The
// y-direction phi is ping-ponged between two buffers (old read from one, new
// written to the other), so the strip-local derivative of the old phi can be
// taken in any band of the bottom pad.
template <int R, int MODE>
__device__ __forceinline__ void bottom_rows(const StepParams& P, const WorkItem& it, float4* ring, int lane) {
    const ShotDev& S = P.shots[it.shot];
    const int pitch = S.pitch, dn = S.dn, nyt = S.nyt;
    const int x0 = it.tile * TILE, xl = x0 + 4 * lane;
    const float* PC = S.pf[P.rp];
    const float* P1 = S.pf[P.rp1];
    float* PO = S.pf[P.wo];
    const float* PHO = P.parity ? S.phy2 : S.phy;  // old y-phi
    float* PHN = P.parity ? S.phy : S.phy2;        // new y-phi
    const int yb0 = nyt - dn;
    const int j0 = it.y0 - yb0, j1 = it.y1 - yb0;
    const int jA = max(j0, R), jB = min(j1 - 1, dn - 1 - R);  // rows with an unclamped phi derivative
    const bool has_hl = (lane == 0) && (x0 > 0), has_hr = (lane == 31) && (x0 + TILE < pitch);
    // this lane stores its elements [lo, hi): the interior columns [sl, sr)
    const int lo = S.off + S.sl - xl, hi = S.off + S.sr - xl;
    const bool full = lo <= 0 && hi >= 4;

    auto issue = [&](int jl, int slot) {
        float4* st = ring + slot * SB_SIZE;
        const int y = yb0 + jl;
        const size_t ro = (size_t)y * pitch + xl;
        if (y + R <= nyt - 1) cp16(st + SB_P + lane, PC + (size_t)(y + R) * pitch + xl);
        cp16(st + SB_P1 + lane, P1 + ro);
        cp16(st + SB_C2 + lane, S.c2 + ro);
        cp16(st + SB_PY + lane, PHO + ro);
        cp16(st + SB_CY + lane, S.chy + ro);
        if (jl >= jA && jl <= jB) cp16(st + SB_FA + lane, PHO + (size_t)(yb0 + jl + R) * pitch + xl);
        if (has_hl) cp16(st + SB_HL, PC + (size_t)y * pitch + x0 - 4);
        if (has_hr) cp16(st + SB_HR, PC + (size_t)y * pitch + x0 + TILE);
    };
#pragma unroll
    for (int i = 0; i < BOT_DEPTH; ++i) {
        if (j0 + i < j1) issue(j0 + i, i);
        cp_commit();
    }

    // the p and old y-phi queues, loaded first so that their latency
    // overlaps the clamp loads below
    float4 q[2 * R + 1], f[2 * R + 1];
#pragma unroll
    for (int i = 0; i < 2 * R; ++i) {
        const int yq = yb0 + j0 - R + i;
        q[i] = (yq <= nyt - 1) ? ldg4(PC + (size_t)yq * pitch + xl) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (jA <= jB) {
#pragma unroll
        for (int i = 0; i < 2 * R; ++i) f[i] = ld4(PHO + (size_t)(yb0 + jA - R + i) * pitch + xl);
    }

    // clamped values: rows jl < R use the phi derivative at local row R, rows
    // jl > dn-1-R that at dn-1-R (solver_space_derivs.f90:118-128 on the
    // strip); rows below nyt-1-R use the p derivatives of row nyt-1-R.  The
    // latter two are the row loop's own derivatives at local row dn-1-R
    // (row nyt-1-R): a band that holds that row takes them there; other
    // bands compute them here.
    const bool bot_clamp = j1 - 1 > dn - 1 - R, bot_in_loop = bot_clamp && j0 <= dn - 1 - R;
    float4 t[2 * R + 1];
    float dphyTop[4] = {0.f, 0.f, 0.f, 0.f}, dphyBot[4] = {0.f, 0.f, 0.f, 0.f};
    float d2yBot[4] = {0.f, 0.f, 0.f, 0.f}, dyBot[4] = {0.f, 0.f, 0.f, 0.f};
    if (j0 < R) {
#pragma unroll
        for (int i = 0; i <= 2 * R; ++i) t[i] = ld4(PHO + (size_t)(yb0 + i) * pitch + xl);
        yderiv1<R>(t, P, dphyTop);
    }
    if (bot_clamp && !bot_in_loop) {
#pragma unroll
        for (int i = 0; i <= 2 * R; ++i) t[i] = ld4(PHO + (size_t)(nyt - 1 - 2 * R + i) * pitch + xl);
        yderiv1<R>(t, P, dphyBot);
#pragma unroll
        for (int i = 0; i <= 2 * R; ++i) t[i] = ldg4(PC + (size_t)(nyt - 1 - 2 * R + i) * pitch + xl);
        yderivs<R>(t, P, d2yBot, dyBot);
    }

    int ri = it.r0;
    int rrow = (ri < it.r1) ? P.recs[ri].row : INT_MAX;
    float2 c1p[R + 1], c2p[R + 1];
#pragma unroll
    for (int i = 0; i <= R; ++i) {
        c1p[i] = make_float2(P.c1[i], P.c1[i]);
        c2p[i] = make_float2(P.c2[i], P.c2[i]);
    }

    // the row's CPML factor, fetched one row ahead
    float An = __ldg(P.fA + j0), Bn = __ldg(P.fB + j0);
    int slot = 0;
    for (int jl = j0; jl < j1; ++jl) {
        const int y = yb0 + jl;
        // bottom strip: factor(j)  (solver_PML_coeffs.f90, pml_matrices_y)
        const float A = An, B = Bn;
        if (jl + 1 < j1) {
            An = __ldg(P.fA + jl + 1);
            Bn = __ldg(P.fB + jl + 1);
        }
        cp_wait<BOT_DEPTH - 1>();
        const float4* st = ring + slot * SB_SIZE;
        if (y + R <= nyt - 1) q[2 * R] = st[SB_P + lane];
        const size_t ro = (size_t)y * pitch + xl;
        const float4 PM1 = st[SB_P1 + lane], CC = st[SB_C2 + lane], PHY = st[SB_PY + lane], CHY = st[SB_CY + lane];
        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 hl = has_hl ? st[SB_HL] : z4, hr = has_hr ? st[SB_HR] : z4;
        float w[12];
        window(q[R], hl, hr, lane, w);
        // strip-local y derivative of the old y-direction phi (pml_matrices_y
        // :335): clamped to local rows R and dn-1-R at the strip's ends
        const int dmode = (jl < R) ? 0 : ((jl <= dn - 1 - R) ? 1 : 2);
        if (dmode == 1) f[2 * R] = st[SB_FA + lane];
        const bool yclamp = y > nyt - 1 - R;
        const float2 Ap = make_float2(A, A), Bp = make_float2(B, B);
        float phy[4], chy[4], p3[4];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            // space_deriv2y / space_derivy: s2 = s2 + (p(j+i)+p(j-i))*c2(i),
            // s1 = s1 + (p(j+i)-p(j-i))*c1(i); rows below nyt-1-R take row nyt-1-R's
            float2 d2y, dy;
            if (!yclamp) {
                float2 s2 = make_float2(0.f, 0.f), s1 = make_float2(0.f, 0.f);
#pragma unroll
                for (int i = 0; i <= R; ++i) {
                    const float2 up = pr(q[R + i], k), dn2 = pr(q[R - i], k);
                    s2 = __fadd2_rn(s2, mul0(__fadd2_rn(up, dn2), c2p[i]));
                    s1 = __fadd2_rn(s1, mul0(__fadd2_rn(up, make_float2(-dn2.x, -dn2.y)), c1p[i]));
                }
                d2y = s2;
                dy = s1;
            } else {
                d2y = make_float2(d2yBot[2 * k], d2yBot[2 * k + 1]);
                dy = make_float2(dyBot[2 * k], dyBot[2 * k + 1]);
            }
            // space_deriv2x: s2 = s2 + c2(i)*(p(j+i)+p(j-i)) (interior columns: no clamp)
            float2 d2x = make_float2(0.f, 0.f);
#pragma unroll
            for (int i = 0; i <= R; ++i) {
                const int ia = 4 + 2 * k + i, ib = 4 + 2 * k - i;
                d2x = __fadd2_rn(d2x, mul0(c2p[i], __fadd2_rn(make_float2(w[ia], w[ia + 1]), make_float2(w[ib], w[ib + 1]))));
            }
            float2 dph;
            if (dmode == 0) {
                dph = make_float2(dphyTop[2 * k], dphyTop[2 * k + 1]);
            } else if (dmode == 1) {
                float2 s1 = make_float2(0.f, 0.f);
#pragma unroll
                for (int i = 0; i <= R; ++i) {
                    const float2 up = pr(f[R + i], k), dn2 = pr(f[R - i], k);
                    s1 = __fadd2_rn(s1, mul0(__fadd2_rn(up, make_float2(-dn2.x, -dn2.y)), c1p[i]));
                }
                dph = s1;
            } else {
                dph = make_float2(dphyBot[2 * k], dphyBot[2 * k + 1]);
            }
            if (bot_in_loop && jl == dn - 1 - R) {  // the clamp values of the rows below
                d2yBot[2 * k] = d2y.x;
                d2yBot[2 * k + 1] = d2y.y;
                dyBot[2 * k] = dy.x;
                dyBot[2 * k + 1] = dy.y;
                dphyBot[2 * k] = dph.x;
                dphyBot[2 * k + 1] = dph.y;
            }
            // phi' = A phi + B dy, chi' = A chi + B (d2y + dphi), prop = dphi + chi',
            // p_3 = (-p_1 + 2p) + c2 ((d2x + d2y) + prop)
            const float2 phyn = __fadd2_rn(mul0(Ap, pr(PHY, k)), mul0(Bp, dy));
            const float2 chyn = __fadd2_rn(mul0(Ap, pr(CHY, k)), mul0(Bp, __fadd2_rn(d2y, dph)));
            const float2 propy = __fadd2_rn(dph, chyn);
            const float2 pc = pr(q[R], k), pm = pr(PM1, k);
            const float2 base = __fadd2_rn(make_float2(-pm.x, -pm.y), __fadd2_rn(pc, pc));
            const float2 r = __fadd2_rn(base, mul0(pr(CC, k), __fadd2_rn(__fadd2_rn(d2x, d2y), propy)));
            phy[2 * k] = phyn.x;
            phy[2 * k + 1] = phyn.y;
            chy[2 * k] = chyn.x;
            chy[2 * k + 1] = chyn.y;
            p3[2 * k] = r.x;
            p3[2 * k + 1] = r.y;
        }
        if (dmode == 1) {
#pragma unroll
            for (int i = 0; i < 2 * R; ++i) f[i] = f[i + 1];
        }
        if (full) {
            st4(PHN + ro, from_arr(phy));
            st4(S.chy + ro, from_arr(chy));
            st4(PO + ro, from_arr(p3));
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (e >= lo && e < hi) {
                    PHN[ro + e] = phy[e];
                    S.chy[ro + e] = chy[e];
                    PO[ro + e] = p3[e];
                }
        }
        if (MODE == 0 && P.record) record_row(P, S, y, xl, ri, it.r1, rrow, p3);

#pragma unroll
        for (int i = 0; i < 2 * R; ++i) q[i] = q[i + 1];
        if (jl + BOT_DEPTH < j1) issue(jl + BOT_DEPTH, slot);
        cp_commit();
        slot = (slot + 1 == BOT_DEPTH) ? 0 : slot + 1;
    }
    cp_wait<0>();
}

template <int R>
__device__ __forceinline__ void interior_update2(const float4* q, float4 L, float4 Rt, float4 pm1, float4 cc,
                                                 const float* sv, const float2* cp, float* p3);

// The same update with the 2R+1 rows given by an accessor: q(i) is row y-R+i.
// The centre terms of both derivatives and the 2p term are the same rounded
// sum p + p; each derivative sum starts from its centre product (the
// reference adds it to 0, which changes nothing but the sign of a zero).
// x-neighbour pairs at odd offsets straddle two register pairs: their sums
// are formed with two scalar adds straight into a pair.
template <int R, typename QF>
__device__ __forceinline__ void interior_update2f(QF q, float4 L, float4 Rt, float4 pm1, float4 cc, const float* sv,
                                                  const float2* cp, float* p3) {
    const float4 C = q(R);
    const float w[12] = {L.x, L.y, L.z, L.w, C.x, C.y, C.z, C.w, Rt.x, Rt.y, Rt.z, Rt.w};
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const float2 pc = pr(C, k);
        const float2 p2 = __fadd2_rn(pc, pc);  // p(j) + p(j)
        const float2 c0 = mul0(cp[0], p2);     // centre term, x and y alike
        // space_deriv2x: s = s + coef(i)*(p(j+i) + p(j-i))
        float2 ax = c0;
#pragma unroll
        for (int i = 1; i <= R; ++i) {
            const int a = 4 + 2 * k + i, b = 4 + 2 * k - i;
            const float2 sx = (i & 1) ? make_float2(w[a] + w[b], w[a + 1] + w[b + 1])
                                      : __fadd2_rn(make_float2(w[a], w[a + 1]), make_float2(w[b], w[b + 1]));
            ax = __fadd2_rn(ax, mul0(cp[i], sx));
        }
        // space_deriv2y: s = s + (p(j+i) + p(j-i))*coef(i)
        float2 ay = c0;
#pragma unroll
        for (int i = 1; i <= R; ++i) ay = __fadd2_rn(ay, mul0(__fadd2_rn(pr(q(R + i), k), pr(q(R - i), k)), cp[i]));
        // p_3 = -p_1 + 2p + (d2x + d2y + source)*c2
        const float2 pm = pr(pm1, k);
        const float2 t = __fadd2_rn(make_float2(-pm.x, -pm.y), p2);
        const float2 u = mul0(__fadd2_rn(__fadd2_rn(ax, ay), make_float2(sv[2 * k], sv[2 * k + 1])), pr(cc, k));
        const float2 r = __fadd2_rn(t, u);
        p3[2 * k] = r.x;
        p3[2 * k + 1] = r.y;
    }
}

template <int R>
__device__ __forceinline__ void interior_update2(const float4* q, float4 L, float4 Rt, float4 pm1, float4 cc,
                                                 const float* sv, const float2* cp, float* p3) {
    interior_update2f<R>([&](int i) { return q[i]; }, L, Rt, pm1, cc, sv, cp, p3);
}

// Model rows, interior columns [sl, sr): no CPML and no clamp, so only
// second derivatives are needed.  The first and last tile of the range may
// be partial; their lanes outside it compute but store nothing (those cells
// belong to the strip warps).  This is the kernel that moves
// almost all of the bytes.  SNAP selects the variant for the time steps
// that store a snapshot (forward) or apply the imaging condition (adjoint);
// the adjoint variant also prefetches the snapshot row and the imaging
// accumulator row through the ring.
constexpr int IN_P = 0, IN_P1 = 32, IN_C2 = 64, IN_HL = 96, IN_HR = 97, IN_F = 98, IN_FS = 130, IN_K = 131;
constexpr int IN_SIZE = 98, IN_SIZE_IMG = 195;
constexpr int IN_DEPTH = 6, IN_DEPTH_IMG = 4;
constexpr int IN_LINE = 34;  // per warp after its ring: injected values / p_3 of a row, [1 + lane]
constexpr int IN_SMEM = 4 * (IN_DEPTH * IN_SIZE + IN_LINE) * 16;
constexpr int IN_SMEM_IMG = 4 * (IN_DEPTH_IMG * IN_SIZE_IMG + IN_LINE) * 16;

__device__ __forceinline__ void cp4(void* smem_dst, const void* gmem_src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp8(void* smem_dst, const void* gmem_src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(gmem_src) : "memory");
}

// Interior item `wid` of the list P.items, run by one warp (w: the warp's
// index in its block, smem: the block's shared memory).
template <int R, int MODE, bool SNAP>
__device__ __forceinline__ void interior_rows(const StepParams& P, int wid, int w, float4* smem) {
    constexpr bool IMG = (MODE == 1) && SNAP;
    constexpr int SZ = IMG ? IN_SIZE_IMG : IN_SIZE;
    constexpr int DEPTH = IMG ? IN_DEPTH_IMG : IN_DEPTH;
    const int lane = threadIdx.x & 31;
    if (wid >= P.nitems) return;
    float4* ring = smem + w * (DEPTH * SZ + IN_LINE);
    float4* line = ring + DEPTH * SZ;
    const WorkItem it = P.items[wid];
    const ShotDev& S = P.shots[it.shot];
    const int pitch = S.pitch;
    const int x0 = it.tile * TILE, xl = x0 + 4 * lane;
    const float* PC = S.pf[P.rp] + xl;   // p at this lane's columns
    const float* P1 = S.pf[P.rp1] + xl;  // p_1
    float* PO = S.pf[P.wo] + xl;         // p_3 (may be the p_1 buffer: each cell reads only its own p_1)
    const float* C2 = S.c2 + xl;
    // lanes 0 and 31 fetch the halo float4 left and right of the tile (in the
    // first and last tile of a row these are the ends of the neighbouring
    // rows: in bounds, and read only by lanes whose columns are outside [sl, sr))
    const int hoff = (lane == 0) ? -4 - 4 * lane : TILE - 4 * lane;
    const bool has_h = (lane == 0) || (lane == 31);
    float4* hslot = ring + (lane == 0 ? IN_HL : IN_HR);
    const size_t snap_base = IMG ? (size_t)P.snap * (size_t)S.snap_stride : 0;
    // this lane stores its elements [lo, hi): the interior columns [sl, sr)
    const int lo = S.off + S.sl - xl, hi = S.off + S.sr - xl;
    const bool full = lo <= 0 && hi >= 4;

    auto issue = [&](int y, int slot) {
        float4* st = ring + slot * SZ;
        const size_t ro = (size_t)y * pitch;
        cp16(st + IN_P + lane, PC + ro + (size_t)R * pitch);
        cp16(st + IN_P1 + lane, P1 + ro);
        cp16(st + IN_C2 + lane, C2 + ro);
        if (has_h) cp16(hslot + slot * SZ, PC + ro + hoff);
        if (IMG) {
            const size_t fo = snap_base + (size_t)(y - S.dn) * pitch + x0;  // element offset of the row segment
            if (P.snap_form == 0) {
                cp16(st + IN_F + lane, reinterpret_cast<const float*>(S.snaps) + fo + 4 * lane);
            } else {
                if (lane < 16) cp16(st + IN_F + lane, reinterpret_cast<const unsigned short*>(S.snaps) + fo + 8 * lane);
                if (lane == 16)
                    cp4(st + IN_FS, S.sscale + ((size_t)P.snap * S.ny + (y - S.dn)) * (S.ntiles + 2) + it.tile);
            }
            const size_t ko = (size_t)(y - S.dn) * pitch + xl;
            if (P.grad_form == 0) {
                cp16(st + IN_K + lane, S.k32 + ko);
            } else {
                cp16(st + IN_K + 2 * lane, S.k64 + ko);
                cp16(st + IN_K + 2 * lane + 1, S.k64 + ko + 2);
            }
        }
    };
#pragma unroll
    for (int i = 0; i < DEPTH; ++i) {
        if (it.y0 + i < it.y1) issue(it.y0 + i, i);
        cp_commit();
    }
    float4 q[2 * R + 1];
#pragma unroll
    for (int i = 0; i < 2 * R; ++i) q[i] = ldg4(PC + (size_t)(it.y0 - R + i) * pitch);

    int si = it.s0, ri = it.r0;
    int srow = (si < it.s1) ? P.srcs[si].row : INT_MAX;
    int rrow = (ri < it.r1) ? P.recs[ri].row : INT_MAX;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float2 cp[R + 1];
#pragma unroll
    for (int i = 0; i <= R; ++i) cp[i] = make_float2(P.c2[i], P.c2[i]);

    int slot = 0;
    for (int y = it.y0; y < it.y1; ++y) {
        cp_wait<DEPTH - 1>();
        const float4* st = ring + slot * SZ;
        q[2 * R] = st[IN_P + lane];
        float pm1[4], cc[4], pc[4];
        to_arr(st[IN_P1 + lane], pm1);
        to_arr(st[IN_C2 + lane], cc);
        to_arr(q[R], pc);
        const float4 h = has_h ? st[lane == 0 ? IN_HL : IN_HR] : z4;
        float4 Lf = shfl_up4(q[R]), Rf = shfl_dn4(q[R]);
        if (lane == 0) Lf = h;
        if (lane == 31) Rf = h;

        // source injection: source(nys,nxs) = S(k-1,j)  (solver_acoustic_SS.f90:319-330)
        float sv[4] = {0.f, 0.f, 0.f, 0.f};
        if (srow == y) to_arr(gather_sources(P, S, y, x0, P.t, si, it.s1, srow, line, lane), sv);
        // p_3 = -p_1 + 2p + (d2x + d2y + source)*c2  (:433-434)
        float p3[4];
        interior_update2<R>(q, Lf, Rf, from_arr(pm1), from_arr(cc), sv, cp, p3);

        if (MODE == 0 && SNAP) store_snapshot(P, S, y - S.dn, lane, xl, lo, hi, p3, pm1, it.tile);
        if (IMG) {
            // kernel += -0.5*(p_3-p_1)*Fields(snap)*store_snap  (:465-466)
            float F[4];
            if (P.snap_form == 0) {
                to_arr(st[IN_F + lane], F);
            } else {
                const uint2 pk = reinterpret_cast<const uint2*>(st + IN_F)[lane];
                const float sc = reinterpret_cast<const float*>(st + IN_FS)[0];
                const unsigned short hv[4] = {(unsigned short)(pk.x & 0xffffu), (unsigned short)(pk.x >> 16),
                                              (unsigned short)(pk.y & 0xffffu), (unsigned short)(pk.y >> 16)};
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    float f;
                    if (P.snap_form == 1) f = __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(&hv[e]));
                    else f = __half2float(*reinterpret_cast<const __half*>(&hv[e]));
                    F[e] = f * sc;
                }
            }
            float k2[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) k2[e] = -(((0.5f * (p3[e] - pm1[e])) * F[e]) * P.ss);
            const size_t ko = (size_t)(y - S.dn) * pitch + xl;
            if (P.grad_form == 0) {
                float4 k = st[IN_K + lane];
                k.x = k.x + k2[0]; k.y = k.y + k2[1]; k.z = k.z + k2[2]; k.w = k.w + k2[3];
                if (full) {
                    st4(S.k32 + ko, k);
                } else {
                    float kv[4];
                    to_arr(k, kv);
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        if (e >= lo && e < hi) S.k32[ko + e] = kv[e];
                }
            } else {
                const double2* kk = reinterpret_cast<const double2*>(st + IN_K) + 2 * lane;
                double2 a = kk[0], b = kk[1];
                a.x += (double)k2[0]; a.y += (double)k2[1]; b.x += (double)k2[2]; b.y += (double)k2[3];
                if (full) {
                    double2* K2 = reinterpret_cast<double2*>(S.k64 + ko);
                    K2[0] = a;
                    K2[1] = b;
                } else {
                    const double kv[4] = {a.x, a.y, b.x, b.y};
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        if (e >= lo && e < hi) S.k64[ko + e] = kv[e];
                }
            }
        }
        if (full) {
            st4(PO + (size_t)y * pitch, from_arr(p3));
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (e >= lo && e < hi) PO[(size_t)y * pitch + e] = p3[e];
        }
        // receivers: every receiver in this cell gets p_3 (:551-555)
        if (MODE == 0 && P.record && rrow == y) {
            line[1 + lane] = from_arr(p3);
            __syncwarp();
            record_row_par(P, S, y, x0, P.t, ri, it.r1, rrow, line, lane);
            __syncwarp();
        }

#pragma unroll
        for (int i = 0; i < 2 * R; ++i) q[i] = q[i + 1];
        if (y + DEPTH < it.y1) issue(y + DEPTH, slot);
        cp_commit();
        slot = (slot + 1 == DEPTH) ? 0 : slot + 1;
    }
    cp_wait<0>();
}

template <int R, int MODE, bool SNAP>
__global__ void __launch_bounds__(128, (MODE == 1 && SNAP) ? 3 : 5) k_step_interior(const __grid_constant__ StepParams P) {
    extern __shared__ float4 smem[];
    const int w = threadIdx.x >> 5;
    interior_rows<R, MODE, SNAP>(P, blockIdx.x * 4 + w, w, smem);
}

// ---------------------------------------------------------------------------
// Side strips: the logical columns [0, sl) and [sr, nxt), in the model rows
// (x-CPML strips, kind 2) and in the bottom pad rows (the corners and the
// y-CPML columns next to them, kind 3).  One warp per band of rows; lane l
// holds the strip-local columns j = 32k + l (k < K), so the CPML arithmetic
// runs once per strip column.  Rows live in shared-memory lines of 32K
// columns plus M margin columns on either side, and every neighbour of a
// cell, in x or y, is a plain shared load:
//   p ring     QN lines, p row r in line r mod QN, with its halo columns;
//   y-phi ring QN lines, the old y-phi row r (bottom rows);
//   row slots  NA slots of NS lines: p_1, c2, x-phi, x-chi, y-chi of row y
//              in slot y mod NA.
// At step y the rings hold rows y-R..y+R and the slot of row y; LA rows
// ahead are in flight (cp.async, 4 bytes per lane and column; every lane
// waits for its own copies, then the warp synchronises before it reads the
// other lanes' columns).
// ---------------------------------------------------------------------------
template <int R, int K>
struct StripLayout {
    static constexpr int M = 4;  // margin columns (>= R; keeps lines 16-byte multiples)
    static constexpr int LINE = 32 * K + 2 * M;
    static constexpr int LA = 4;  // rows of lookahead
    static constexpr int QN = 2 * R + 1 + LA;
    static constexpr int NA = LA + 1;
    static constexpr int S_P1 = 0, S_C2 = 1, S_PX = 2, S_CX = 3, S_CY = 4, NS = 5;
    static constexpr int P_RING = 0, Y_RING = QN * LINE, SLOTS = 2 * QN * LINE;
    static constexpr int WARP = SLOTS + NA * NS * LINE;  // floats per warp
};
template <int R, int K>
constexpr int strip_smem() {
    return 4 * StripLayout<R, K>::WARP * 4;
}

// Value at the warp-uniform strip-local column j of a per-lane array.
template <int K>
__device__ __forceinline__ float bcast(const float (&v)[K], int j) {
    const float src = (K > 1 && j >= 32) ? v[K - 1] : v[0];
    return __shfl_sync(FULL, src, j & 31);
}

template <int R, int MODE, int K, bool BOT>
__device__ __forceinline__ void strip_rows(const StepParams& P, const WorkItem& it, float* sw, int lane) {
    using L = StripLayout<R, K>;
    const ShotDev& S = P.shots[it.shot];
    const int pitch = S.pitch, dn = S.dn, nx = S.nx, nxt = S.nxt, nyt = S.nyt;
    const bool right = it.tile != 0;
    const int cs = right ? S.sr : 0, ce = right ? nxt : S.sl;  // logical strip columns [cs, ce)
    const float* PC = S.pf[P.rp];   // p
    const float* P1 = S.pf[P.rp1];  // p_1
    float* PO = S.pf[P.wo];         // p_3
    const float* PHO = P.parity ? S.phy2 : S.phy;  // old y-phi (bottom rows)
    float* PHN = P.parity ? S.phy : S.phy2;        // new y-phi
    const int yb0 = nyt - dn;
    const size_t xs = (size_t)S.off + cs;  // physical column of strip column 0

    int col[K];
    bool valid[K], act[K], xc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        col[k] = cs + 32 * k + lane;
        valid[k] = col[k] < nxt;  // inside the grid (a neighbour of some cell)
        act[k] = col[k] < ce;     // updated by this warp
        xc[k] = act[k] && (col[k] < dn || col[k] >= dn + nx);  // x-CPML column
    }
    // halo columns, copied by lanes 0..R-1: left j = lane-R, right j = 32K+lane
    const int jhl = lane - R, jhr = 32 * K + lane;
    const bool has_hl = lane < R && cs + jhl >= 0, has_hr = lane < R && cs + jhr < nxt;

    float* pring = sw + L::P_RING;
    float* yring = sw + L::Y_RING;
    float* slots = sw + L::SLOTS;
    // ring positions: padded row r lives in line r % QN of the p / y-phi
    // rings and row y's per-cell inputs in slot y % NA; the row loop keeps
    // both positions incrementally (rows are >= 0: every item starts at or
    // below row dn >= R)
    auto pline = [&](int q) { return pring + q * L::LINE + L::M; };
    auto yline = [&](int q) { return yring + q * L::LINE + L::M; };
    auto sline = [&](int q, int f) { return slots + (q * L::NS + f) * L::LINE + L::M; };

    // p row r (and the old y-phi row r) into ring line q; rows past the grid
    // are never read
    auto issue_row = [&](int r, int q) {
        if (r > nyt - 1) return;
        float* d = pline(q);
        const float* src = PC + (size_t)r * pitch + xs;
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (valid[k]) cp4(d + 32 * k + lane, src + 32 * k + lane);
        if (has_hl) cp4(d + jhl, src + jhl);
        if (has_hr) cp4(d + jhr, src + jhr);
        if (BOT && r >= yb0) {
            float* e = yline(q);
            const float* ysrc = PHO + (size_t)r * pitch + xs;
#pragma unroll
            for (int k = 0; k < K; ++k)
                if (valid[k]) cp4(e + 32 * k + lane, ysrc + 32 * k + lane);
        }
    };
    auto issue_slot = [&](int y, int q) {
        const size_t ro = (size_t)y * pitch + xs;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int j = 32 * k + lane;
            if (act[k]) {
                cp4(sline(q, L::S_P1) + j, P1 + ro + j);
                cp4(sline(q, L::S_C2) + j, S.c2 + ro + j);
                if (BOT) cp4(sline(q, L::S_CY) + j, S.chy + ro + j);
            }
            if (xc[k]) {
                cp4(sline(q, L::S_PX) + j, S.phx + ro + j);
                cp4(sline(q, L::S_CX) + j, S.chx + ro + j);
            }
        }
    };
    const int y0 = it.y0, y1 = it.y1;
#pragma unroll 1
    for (int i = 0; i < 2 * R; ++i) issue_row(y0 - R + i, (y0 - R + i) % L::QN);
    cp_commit();
#pragma unroll 1
    for (int i = 0; i < L::LA; ++i) {
        if (y0 + i < y1) {
            issue_row(y0 + i + R, (y0 + i + R) % L::QN);
            issue_slot(y0 + i, (y0 + i) % L::NA);
        }
        cp_commit();
    }

    // clamp sources (warp-uniform strip-local columns): the p derivatives of
    // columns < R copy column R, of columns > nxt-1-R column nxt-1-R
    // (solver_space_derivs.f90:18-23, :84-94); the strip-local derivative of
    // the old x-phi copies its value at strip index R / dn-1-R
    // (solver_PML_matrices.f90:15, :97 on the dn-wide strip array).
    const int jc = right ? (nxt - 1 - R - cs) : R;
    const int jlo = right ? (dn + nx + R - cs) : R;
    const int jhi = right ? (nxt - 1 - R - cs) : (dn - 1 - R);

    // bottom rows: the y-phi derivative of rows jl < R is that of row R, of
    // rows jl > dn-1-R that of row dn-1-R; rows below nyt-1-R take the p
    // derivatives of row nyt-1-R (solver_space_derivs.f90:38-53, :109-128)
    float dphyTop[K], dphyBot[K], d2yBot[K], dyBot[K];
#pragma unroll
    for (int k = 0; k < K; ++k) dphyTop[k] = dphyBot[k] = d2yBot[k] = dyBot[k] = 0.f;
    if (BOT) {
        const int j0 = y0 - yb0, j1 = y1 - yb0;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if (!valid[k]) continue;
            const size_t cx = xs + 32 * k + lane;
            if (j0 < R) {
                float s1 = 0.f;
#pragma unroll
                for (int i = 0; i <= R; ++i)
                    s1 = s1 + (PHO[(size_t)(yb0 + R + i) * pitch + cx] - PHO[(size_t)(yb0 + R - i) * pitch + cx]) * P.c1[i];
                dphyTop[k] = s1;
            }
            if (j1 - 1 > dn - 1 - R) {
                const int yc = nyt - 1 - R;
                float s1 = 0.f, s2 = 0.f, t1 = 0.f;
#pragma unroll
                for (int i = 0; i <= R; ++i) {
                    s1 = s1 + (PHO[(size_t)(yc + i) * pitch + cx] - PHO[(size_t)(yc - i) * pitch + cx]) * P.c1[i];
                    const float a = __ldg(PC + (size_t)(yc + i) * pitch + cx), b = __ldg(PC + (size_t)(yc - i) * pitch + cx);
                    s2 = s2 + (a + b) * P.c2[i];
                    t1 = t1 + (a - b) * P.c1[i];
                }
                dphyBot[k] = s1;
                d2yBot[k] = s2;
                dyBot[k] = t1;
            }
        }
    }
    float2 c1p[R + 1], c2p[R + 1];
#pragma unroll
    for (int i = 0; i <= R; ++i) {
        c1p[i] = make_float2(P.c1[i], P.c1[i]);
        c2p[i] = make_float2(P.c2[i], P.c2[i]);
    }

    int si = it.s0, ri = it.r0;
    int srow = (si < it.s1) ? P.srcs[si].row : INT_MAX;
    int rrow = (ri < it.r1) ? P.recs[ri].row : INT_MAX;
    const size_t seg = (size_t)S.ntiles + (right ? 1 : 0);

    // CPML factor index of each lane's column: per column in the model rows
    // (xl strip: factor(dn-i+1), xr strip: factor(i), solver_PML_matrices.f90:296-312);
    // in the bottom rows factor(j), in the corners factor(max(i,j)) with the
    // ld/rd orientation (solver_PML_coeffs.f90:240-267).  The factors of a
    // row are fetched one row ahead.
    int cfi[K];
#pragma unroll
    for (int k = 0; k < K; ++k) cfi[k] = xc[k] ? ((col[k] < dn) ? (dn - 1 - col[k]) : (col[k] - dn - nx)) : 0;
    auto fidx = [&](int k, int jrow) {
        if (!BOT) return cfi[k];
        int fi = jrow;
        if (xc[k]) fi = max(jrow, cfi[k]);
        if (!act[k]) fi = 0;
        return fi;
    };
    float fa[K], fb[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int fi = fidx(k, BOT ? y0 - yb0 : 0);
        fa[k] = __ldg(P.fA + fi);
        fb[k] = __ldg(P.fB + fi);
    }

    int qy = y0 % L::QN, sy = y0 % L::NA;  // ring line of row y, slot of row y
    // ring line of row y + i for a compile-time i in [-QN, QN]
    auto qat = [&](int i) {
        int q = qy + i;
        if (i > 0) q = (q >= L::QN) ? q - L::QN : q;
        if (i < 0) q = (q < 0) ? q + L::QN : q;
        return q;
    };
#pragma unroll 1
    for (int y = y0; y < y1; ++y) {
        float ca[K], cb[K];  // this row's factors
#pragma unroll
        for (int k = 0; k < K; ++k) {
            ca[k] = fa[k];
            cb[k] = fb[k];
        }
        if (BOT && y + 1 < y1) {
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const int fi = fidx(k, y + 1 - yb0);
                fa[k] = __ldg(P.fA + fi);
                fb[k] = __ldg(P.fB + fi);
            }
        }
        cp_wait<L::LA - 1>();
        __syncwarp();
        const int jl = y - yb0;  // bottom rows: index inside the bottom strip
        const float* pl = pline(qy);
        const float* px = sline(sy, L::S_PX);
        float pc[K], d2x[K], dx[K], d2y[K], dy[K], dphx[K], dphy[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int j = 32 * k + lane;
            pc[k] = pl[j];
            // (d2x, d2y): s2 = s2 + c2(i)*(p(j+i)+p(j-i)), s2 = s2 + (p(j+i)+p(j-i))*c2(i)
            // (dx, dy):   s1 = s1 + (p(j+i)-p(j-i))*c1(i)
            // (dphx, dphy): the same on the old phi
            // space_deriv2x/2y, space_derivx/y (solver_space_derivs.f90:11-16, :38-45, :70-82, :109-116)
            float2 a2 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f), ap = make_float2(0.f, 0.f);
#pragma unroll
            for (int i = 0; i <= R; ++i) {
                const float2 hi_ = make_float2(pl[j + i], pline(qat(i))[j]);
                const float2 lo_ = make_float2(pl[j - i], pline(qat(-i))[j]);
                a2 = __fadd2_rn(a2, mul0(__fadd2_rn(hi_, lo_), c2p[i]));
                a1 = __fadd2_rn(a1, mul0(__fadd2_rn(hi_, make_float2(-lo_.x, -lo_.y)), c1p[i]));
                const float2 fh = make_float2(px[j + i], BOT ? yline(qat(i))[j] : 0.f);
                const float2 fl = make_float2(px[j - i], BOT ? yline(qat(-i))[j] : 0.f);
                ap = __fadd2_rn(ap, mul0(__fadd2_rn(fh, make_float2(-fl.x, -fl.y)), c1p[i]));
            }
            d2x[k] = a2.x;
            d2y[k] = a2.y;
            dx[k] = a1.x;
            dy[k] = a1.y;
            dphx[k] = ap.x;
            dphy[k] = ap.y;
        }
        {
            const float c2v = bcast<K>(d2x, jc), c1v = bcast<K>(dx, jc);
            const float plo = bcast<K>(dphx, jlo), phi_ = bcast<K>(dphx, jhi);
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const int c = col[k];
                if (right ? (c > nxt - 1 - R) : (c < R)) {
                    d2x[k] = c2v;
                    dx[k] = c1v;
                }
                const int il = right ? c - dn - nx : c;  // index inside the dn-wide x-CPML strip
                if (il < R) dphx[k] = plo;
                else if (il > dn - 1 - R) dphx[k] = phi_;
                if (BOT) {
                    if (y > nyt - 1 - R) {
                        d2y[k] = d2yBot[k];
                        dy[k] = dyBot[k];
                    }
                    if (jl < R) dphy[k] = dphyTop[k];
                    else if (jl > dn - 1 - R) dphy[k] = dphyBot[k];
                }
            }
        }

        // source injection: source(nys,nxs) = S(k-1,j), interior cells only
        float sv[K];
#pragma unroll
        for (int k = 0; k < K; ++k) sv[k] = 0.f;
        while (!BOT && srow == y) {
            const SrcEnt e = P.srcs[si];
            const float val = __ldg(S.srcv + (size_t)e.vidx * S.nt + P.t);
#pragma unroll
            for (int k = 0; k < K; ++k)
                if (e.col == (int)xs + 32 * k + lane) sv[k] = val;
            ++si;
            srow = (si < it.s1) ? P.srcs[si].row : INT_MAX;
        }

        float p3[K], pm1[K];
        const size_t ro = (size_t)y * pitch + xs + lane;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int j = 32 * k + lane, c = col[k];
            pm1[k] = sline(sy, L::S_P1)[j];
            const float cc = sline(sy, L::S_C2)[j];
            const float base = (-pm1[k]) + 2.f * pc[k];
            if (!BOT) {
                if (xc[k]) {
                    const float A = ca[k], B = cb[k];
                    const float phn = A * px[j] + B * dx[k];
                    const float chn = A * sline(sy, L::S_CX)[j] + B * (d2x[k] + dphx[k]);
                    const float prop = dphx[k] + chn;
                    p3[k] = base + cc * ((d2x[k] + d2y[k]) + prop);
                    S.phx[ro + 32 * k] = phn;
                    S.chx[ro + 32 * k] = chn;
                } else {
                    p3[k] = base + (((d2x[k] + d2y[k]) + sv[k]) * cc);
                }
            } else {
                const float A = ca[k], B = cb[k];
                const float phyn = A * yline(qy)[j] + B * dy[k];
                const float chyn = A * sline(sy, L::S_CY)[j] + B * (d2y[k] + dphy[k]);
                const float propy = dphy[k] + chyn;
                if (xc[k]) {
                    // corner, two stages (solver_acoustic_SS.f90:395-411)
                    const float phxn = A * px[j] + B * dx[k];
                    const float chxn = A * sline(sy, L::S_CX)[j] + B * (d2x[k] + dphx[k]);
                    const float propx = dphx[k] + chxn;
                    const float tt = base + cc * ((d2x[k] + d2y[k]) + propx);
                    p3[k] = tt + cc * propy;
                    S.phx[ro + 32 * k] = phxn;
                    S.chx[ro + 32 * k] = chxn;
                } else {
                    p3[k] = base + cc * ((d2x[k] + d2y[k]) + propy);
                }
                if (act[k]) {
                    PHN[ro + 32 * k] = phyn;
                    S.chy[ro + 32 * k] = chyn;
                }
            }
        }

        if (!BOT && P.snap >= 0) {
            const int yrow = y - dn;
            const size_t fb = (size_t)P.snap * (size_t)S.snap_stride + (size_t)yrow * pitch + xs + lane;
            bool in[K];
#pragma unroll
            for (int k = 0; k < K; ++k) in[k] = act[k] && !xc[k];
            if (MODE == 0) {
                // Fields(j, snap*nx+i) = (p_3 - p_1)*0.5/dt  (:447)
                float v[K];
#pragma unroll
                for (int k = 0; k < K; ++k) v[k] = in[k] ? div_by_const((p3[k] - pm1[k]) * 0.5f, P.dt, P.rdt) : 0.f;
                if (P.snap_form == 0) {
#pragma unroll
                    for (int k = 0; k < K; ++k)
                        if (in[k]) reinterpret_cast<float*>(S.snaps)[fb + 32 * k] = v[k];
                } else {
                    float m = fabsf(v[0]);
#pragma unroll
                    for (int k = 1; k < K; ++k) m = fmaxf(m, fabsf(v[k]));
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(FULL, m, o));
                    int ex = 0;
                    if (m > 0.f) frexpf(m, &ex);
                    const int sh = 14 - ex;
#pragma unroll
                    for (int k = 0; k < K; ++k) {
                        if (!in[k]) continue;
                        const float scaled = ldexpf(v[k], sh);
                        unsigned short h;
                        if (P.snap_form == 1) {
                            __nv_bfloat16 b = __float2bfloat16_rn(scaled);
                            h = *reinterpret_cast<unsigned short*>(&b);
                        } else {
                            __half b = __float2half_rn(scaled);
                            h = *reinterpret_cast<unsigned short*>(&b);
                        }
                        reinterpret_cast<unsigned short*>(S.snaps)[fb + 32 * k] = h;
                    }
                    if (lane == 0) S.sscale[((size_t)P.snap * S.ny + yrow) * (S.ntiles + 2) + seg] = ldexpf(1.f, -sh);
                }
            } else {
                // kernel += -0.5*(p_3-p_1)*Fields(snap)*store_snap  (:465-466)
                const float sc = (P.snap_form == 0)
                                     ? 1.f
                                     : __ldg(S.sscale + ((size_t)P.snap * S.ny + yrow) * (S.ntiles + 2) + seg);
                const size_t ko = (size_t)yrow * pitch + xs + lane;
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    if (!in[k]) continue;
                    float F;
                    if (P.snap_form == 0) {
                        F = __ldg(reinterpret_cast<const float*>(S.snaps) + fb + 32 * k);
                    } else {
                        const unsigned short h = __ldg(reinterpret_cast<const unsigned short*>(S.snaps) + fb + 32 * k);
                        float f;
                        if (P.snap_form == 1) f = __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(&h));
                        else f = __half2float(*reinterpret_cast<const __half*>(&h));
                        F = f * sc;
                    }
                    const float k2 = -(((0.5f * (p3[k] - pm1[k])) * F) * P.ss);
                    if (P.grad_form == 0) S.k32[ko + 32 * k] = S.k32[ko + 32 * k] + k2;
                    else S.k64[ko + 32 * k] += (double)k2;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (act[k]) PO[ro + 32 * k] = p3[k];
        // receivers: every receiver in this cell gets p_3 (:553)
        if (MODE == 0 && P.record) {
            while (rrow == y) {
                const RecEnt r = P.recs[ri];
#pragma unroll
                for (int k = 0; k < K; ++k)
                    if (r.col == (int)xs + 32 * k + lane) S.rec[(size_t)r.ridx * S.nt + P.t] = p3[k];
                ++ri;
                rrow = (ri < it.r1) ? P.recs[ri].row : INT_MAX;
            }
        }

        if (y + L::LA < y1) {
            issue_row(y + L::LA + R, qat(L::LA + R));
            issue_slot(y + L::LA, (sy + L::LA >= L::NA) ? sy + L::LA - L::NA : sy + L::LA);
        }
        cp_commit();
        qy = (qy + 1 == L::QN) ? 0 : qy + 1;
        sy = (sy + 1 == L::NA) ? 0 : sy + 1;
    }
    cp_wait<0>();
}

template <int R, int MODE, int K>
__global__ void __launch_bounds__(128) k_step_strip(const __grid_constant__ StepParams P) {
    extern __shared__ float sfl[];
    const int lane = threadIdx.x & 31;
    const int wid = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (wid >= P.nstrip) return;
    float* sw = sfl + (threadIdx.x >> 5) * StripLayout<R, K>::WARP;
    const WorkItem it = P.items[wid];
    if (it.kind == 3) strip_rows<R, MODE, K, true>(P, it, sw, lane);
    else strip_rows<R, MODE, K, false>(P, it, sw, lane);
}

// ---------------------------------------------------------------------------
// Two time steps of the model-row interior in one pass (temporal blocking).
//
// A two-step tile owns the output columns [x0, x0 + F2_W) of rows [y0, y1).
// Lane l holds the four columns x0 - 4 + 4l, so the warp spans [x0 - 4,
// x0 + 124): the first step (p_{n+1}) is computed on all 128 columns, the
// second (p_{n+2}) on the 120 columns of lanes 1..30, whose x-neighbours
// (R <= 4 columns) are all on the warp.  The first step runs over rows
// [y0 - R, y1 + R] (rows above the model rows are the free-surface pad:
// zero; the last row only keeps the loop uniform), the second R+1 rows
// behind it, so the two updates of one row iteration are independent.  p_n
// comes through a register queue of 2R+2 rows, p_{n+1} through one of 2R+1;
// p_{n-1}, c2 and p_n with its halo float4s through a cp.async ring whose
// slots are kept R+1 rows longer (the x-neighbours of p_n row y sit in the
// slot of row y - R, the second step's c2 in that of row y - R - 1).  The
// x-neighbours of both steps are shared-memory reads from lines laid out
// [halo | 32 lanes | halo]; a row's injected values and recorded receivers go
// through a shared line too, 32 entries at a time.  Both results go to
// buffers other than the inputs (the warp reads its neighbours' p_n and
// p_{n-1}), and the cells a warp computes outside its own columns and rows
// are bit-identical to their owners' (same arithmetic, same source
// injection; the host only makes tiles whose halo cells are plain interior
// cells).
// ---------------------------------------------------------------------------
constexpr int F2_W = 120;
// ring slot of row y: p_n row y+R with its halo float4s [HL | 32 lanes | HR],
// p_{n-1} row y, c2 row y
constexpr int F2_HL = 0, F2_P = 1, F2_HR = 33, F2_P1 = 34, F2_C2 = 66, F2_SIZE = 98;
constexpr int F2_DEPTH = 4;  // rows in flight
constexpr int F2_LINE = 34;  // p_{n+1} line: [garbage | 32 lanes | garbage]
// imaging passes: per row in flight the snapshot row (FP32: 32 float4;
// 16-bit: 16 float4 and one scale per lane) and the accumulator row (FP32: 32
// float4; FP64: 64 float4)
constexpr int F2_IF = 0, F2_IS = 32, F2_IK = 40, F2_ISIZE = 104;
template <int R, bool IMG = false>
struct F2Ring {
    static constexpr int SLOTS = F2_DEPTH + R + 1;
    static constexpr int Q1 = R + 2;  // p_{n+1} lines: rows y-R-1 .. y
    static constexpr int WARP = SLOTS * F2_SIZE + (Q1 + 1) * F2_LINE + (IMG ? F2_DEPTH * F2_ISIZE : 0);  // float4 per warp
    static constexpr int SMEM = 4 * WARP * 16;
};



// SNAP: the first of the two steps stores a snapshot (MODE 0, FP32 form) or
// applies the imaging condition (MODE 1) at the tile's own cells, as
// k_step_interior does at a snapshot step (P.snap = the block).
// Snapshot store (MODE 0: Fields = (p_3 - p_1)*0.5/dt, FP32 form) or imaging
// condition (MODE 1: kernel += -0.5*(p_3-p_1)*Fields*store_snap) for the
// elements [lo, hi) of this lane's four cells in snapshot row yrow, the same
// arithmetic as k_step_interior's snapshot steps (solver_acoustic_SS.f90:447,
// :465-466).  The scale of a 16-bit snapshot is that of the cell's 128-column
// segment.
template <int MODE>
__device__ __forceinline__ void snap_or_image(const StepParams& P, const ShotDev& S, int yrow, int xl, int lo, int hi,
                                              bool full, const float* p3, float4 pm1v, const float4* isl, int lane) {
    float pm1[4];
    to_arr(pm1v, pm1);
    const size_t fo = (size_t)P.snap * (size_t)S.snap_stride + (size_t)yrow * S.pitch + xl;
    if (MODE == 0) {
        float v[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) v[e] = div_by_const((p3[e] - pm1[e]) * 0.5f, P.dt, P.rdt);
        float* F = reinterpret_cast<float*>(S.snaps) + fo;
        if (full) {
            st4(F, from_arr(v));
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (e >= lo && e < hi) F[e] = v[e];
        }
        return;
    }
    // the snapshot and accumulator rows were prefetched into the slot isl
    float F[4];
    if (P.snap_form == 0) {
        to_arr(isl[F2_IF + lane], F);
    } else {
        const uint2 pk = reinterpret_cast<const uint2*>(isl + F2_IF)[lane];
        const float sc = reinterpret_cast<const float*>(isl + F2_IS)[lane];
        const unsigned short hv[4] = {(unsigned short)(pk.x & 0xffffu), (unsigned short)(pk.x >> 16),
                                      (unsigned short)(pk.y & 0xffffu), (unsigned short)(pk.y >> 16)};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            float f;
            if (P.snap_form == 1) f = __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(&hv[e]));
            else f = __half2float(*reinterpret_cast<const __half*>(&hv[e]));
            F[e] = f * sc;
        }
    }
    float k2[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) k2[e] = -(((0.5f * (p3[e] - pm1[e])) * F[e]) * P.ss);
    const size_t ko = (size_t)yrow * S.pitch + xl;
    if (P.grad_form == 0) {
        float kv[4];
        to_arr(isl[F2_IK + lane], kv);
#pragma unroll
        for (int e = 0; e < 4; ++e) kv[e] = kv[e] + k2[e];
        if (full) {
            st4(S.k32 + ko, from_arr(kv));
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (e >= lo && e < hi) S.k32[ko + e] = kv[e];
        }
    } else {
        const double2* kk = reinterpret_cast<const double2*>(isl + F2_IK) + 2 * lane;
        double2 a = kk[0], b = kk[1];
        a.x += (double)k2[0];
        a.y += (double)k2[1];
        b.x += (double)k2[2];
        b.y += (double)k2[3];
        if (full) {
            double2* K2 = reinterpret_cast<double2*>(S.k64 + ko);
            K2[0] = a;
            K2[1] = b;
        } else {
            const double kv[4] = {a.x, a.y, b.x, b.y};
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (e >= lo && e < hi) S.k64[ko + e] = kv[e];
        }
    }
}

template <int R, int MODE, bool SNAP>
__global__ void __launch_bounds__(128, (MODE == 1 && SNAP) ? 2 : 3) k_step2_interior(const __grid_constant__ StepParams P) {
    constexpr bool IMG = MODE == 1 && SNAP;
    using RG = F2Ring<R, IMG>;
    extern __shared__ float4 smem[];
    const int lane = threadIdx.x & 31;
    const int wid = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (wid >= P.nitems) return;
    float4* ring = smem + (threadIdx.x >> 5) * RG::WARP;
    float4* q1l = ring + RG::SLOTS * F2_SIZE;  // p_{n+1} lines
    float4* inj = q1l + RG::Q1 * F2_LINE;       // injected values of a row
    float4* iring = inj + F2_LINE;              // imaging rows (IMG)
    const WorkItem it = P.items[wid];
    const ShotDev& S = P.shots[it.shot];
    const int pitch = S.pitch, dn = S.dn;
    const int x0 = it.tile, xl = x0 - 4 + 4 * lane;
    const float* PN = S.pf[P.rp] + xl;    // p_n
    const float* PM = S.pf[P.rp1] + xl;   // p_{n-1}
    float* O1 = S.pf[P.wo] + xl;          // p_{n+1}
    float* O2 = S.pf[P.wo2] + xl;         // p_{n+2}
    const float* C2 = S.c2 + xl;
    // lanes 0 and 31 also fetch the halo float4 beyond the warp's columns
    const bool has_h = (lane == 0) || (lane == 31);
    const int hslot = (lane == 0) ? F2_HL : F2_HR, hoff = (lane == 0) ? -4 : 4;
    // lanes 1..30 store their elements [lo, hi): the interior columns [sl, sr)
    const int lo = S.off + S.sl - xl, hi = S.off + S.sr - xl;
    const bool mine = lane >= 1 && lane <= 30;
    const bool full = mine && lo <= 0 && hi >= 4, part = mine && !full && lo < 4 && hi > 0;
    // first step over rows [ya, yb) (one row past the R halo rows below, so
    // that the second step, R+1 rows behind, ends at row y1 - 1)
    const int y0 = it.y0, y1 = it.y1, ya = y0 - R, yb = y1 + R + 1;

    auto issue = [&](int y, int slot) {
        float4* st = ring + slot * F2_SIZE;
        const size_t ro = (size_t)y * pitch;
        cp16(st + F2_P + lane, PN + ro + (size_t)R * pitch);
        if (has_h) cp16(st + hslot, PN + ro + (size_t)R * pitch + hoff);
        cp16(st + F2_P1 + lane, PM + ro);
        cp16(st + F2_C2 + lane, C2 + ro);
    };
    // imaging passes: the snapshot and accumulator rows of the own rows, into
    // slot (y - ya) mod DEPTH, with the row's other copies
    auto issue_img = [&](int y, int islot) {
        if (!IMG || y < y0 || y >= y1) return;
        float4* isl = iring + islot * F2_ISIZE;
        const int yrow = y - dn;
        const size_t fo = (size_t)P.snap * (size_t)S.snap_stride + (size_t)yrow * pitch + xl;
        if (P.snap_form == 0) {
            cp16(isl + F2_IF + lane, reinterpret_cast<const float*>(S.snaps) + fo);
        } else {
            cp8(reinterpret_cast<uint2*>(isl + F2_IF) + lane, reinterpret_cast<const unsigned short*>(S.snaps) + fo);
            cp4(reinterpret_cast<float*>(isl + F2_IS) + lane,
                S.sscale + ((size_t)P.snap * S.ny + yrow) * (S.ntiles + 2) + (xl >> 7));
        }
        const size_t ko = (size_t)yrow * pitch + xl;
        if (P.grad_form == 0) {
            cp16(isl + F2_IK + lane, S.k32 + ko);
        } else {
            cp16(isl + F2_IK + 2 * lane, S.k64 + ko);
            cp16(isl + F2_IK + 2 * lane + 1, S.k64 + ko + 2);
        }
    };
    // the x-neighbours of row y's p_n sit in the slot of row y - R, which
    // holds p_n row y (with its halos); for the first R rows these are slots
    // SLOTS-R .. SLOTS-1 (rows ya-R .. ya-1), filled here
    float4* pre = ring + (RG::SLOTS - R) * F2_SIZE;
#pragma unroll
    for (int i = 0; i < R; ++i) {
        const size_t ro = (size_t)(ya + i) * pitch;
        cp16(pre + i * F2_SIZE + F2_P + lane, PN + ro);
        if (has_h) cp16(pre + i * F2_SIZE + hslot, PN + ro + hoff);
    }
    cp_commit();
#pragma unroll
    for (int i = 0; i < F2_DEPTH; ++i) {
        issue(ya + i, i);
        issue_img(ya + i, i);
        cp_commit();
    }
    // qn: p_n rows y-R-1 .. y+R; q1: p_{n+1} rows y-2R-1 .. y-1 (before row y's first step)
    float4 qn[2 * R + 2], q1[2 * R + 1];
#pragma unroll
    for (int i = 0; i < 2 * R + 1; ++i) qn[i] = ldg4(PN + (size_t)(ya - R - 1 + i) * pitch);
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int i = 0; i <= 2 * R; ++i) q1[i] = z4;

    // source cursors: first step from the list start, second step from row y0
    int si1 = it.s0, si2 = it.s0, ri1 = it.r0, ri2 = it.r0;
    while (si2 < it.s1 && P.srcs[si2].row < y0) ++si2;
    int srow1 = (si1 < it.s1) ? P.srcs[si1].row : INT_MAX, srow2 = (si2 < it.s1) ? P.srcs[si2].row : INT_MAX;
    int rrow1 = (ri1 < it.r1) ? P.recs[ri1].row : INT_MAX, rrow2 = rrow1;
    float2 cp[R + 1];
#pragma unroll
    for (int i = 0; i <= R; ++i) cp[i] = make_float2(P.c2[i], P.c2[i]);

    // slot of row y, of row y - R (x-neighbours of p_n row y), of row y - R - 1 (c2 of the second step);
    // p_{n+1} line of row y and of row y - R - 1
    int slot = 0, slotx = RG::SLOTS - R, slot2 = RG::SLOTS - R - 1, l1 = 0, l2 = 1, islot = 0;
    for (int y = ya; y < yb; ++y) {
        // every lane has its own copies of row y (and of the pre slots); the
        // warp synchronises before it reads the other lanes' copies and the
        // p_{n+1} line written R+1 iterations ago
        cp_wait<F2_DEPTH - 1>();
        __syncwarp();
        const float4* st = ring + slot * F2_SIZE;
        const float4* sx = ring + slotx * F2_SIZE;
        qn[2 * R + 1] = st[F2_P + lane];
        // first step, row y: p_{n+1} = -p_{n-1} + 2p_n + (d2x + d2y + source)*c2
        float np1[4] = {0.f, 0.f, 0.f, 0.f};
        {
            const float4 Lf = sx[F2_HL + lane], Rf = sx[F2_P + 1 + lane];
            float sv[4] = {0.f, 0.f, 0.f, 0.f};
            if (srow1 == y) to_arr(gather_sources(P, S, y, x0 - 4, P.t, si1, it.s1, srow1, inj, lane), sv);
            if (y >= dn) interior_update2<R>(qn + 1, Lf, Rf, st[F2_P1 + lane], st[F2_C2 + lane], sv, cp, np1);
        }
        q1l[l1 * F2_LINE + 1 + lane] = from_arr(np1);
        // second step, row y - R - 1, from the p_{n+1} rows of earlier iterations
        // (independent of this iteration's first step)
        const int y2 = y - R - 1;
        if (y2 >= y0) {
            const float4* st2 = ring + slot2 * F2_SIZE;
            const float4* ln = q1l + l2 * F2_LINE;
            const float4 Lf = ln[lane], Rf = ln[lane + 2];
            float sv[4] = {0.f, 0.f, 0.f, 0.f};
            if (srow2 == y2) to_arr(gather_sources(P, S, y2, x0 - 4, P.t + 1, si2, it.s1, srow2, inj, lane), sv);
            float np2[4];
            interior_update2<R>(q1, Lf, Rf, qn[0], st2[F2_C2 + lane], sv, cp, np2);
            if (full) {
                st4(O2 + (size_t)y2 * pitch, from_arr(np2));
            } else if (part) {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (e >= lo && e < hi) O2[(size_t)y2 * pitch + e] = np2[e];
            }
            if (MODE == 0 && P.record && rrow2 == y2) {
                inj[1 + lane] = from_arr(np2);  // the injection line is free again
                __syncwarp();
                record_row_par(P, S, y2, x0 - 4, P.t + 1, ri2, it.r1, rrow2, inj, lane);
            }
        }
        if (y >= y0 && y < y1) {
            if (full) {
                st4(O1 + (size_t)y * pitch, from_arr(np1));
            } else if (part) {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (e >= lo && e < hi) O1[(size_t)y * pitch + e] = np1[e];
            }
            if (MODE == 0 && P.record && rrow1 == y) {
                __syncwarp();  // np1 of every lane is in its p_{n+1} line
                record_row_par(P, S, y, x0 - 4, P.t, ri1, it.r1, rrow1, q1l + l1 * F2_LINE, lane);
            }
            if (SNAP && (full || part))
                snap_or_image<MODE>(P, S, y - dn, xl, lo, hi, full, np1, st[F2_P1 + lane], iring + islot * F2_ISIZE,
                                    lane);
        }
#pragma unroll
        for (int i = 0; i < 2 * R + 1; ++i) qn[i] = qn[i + 1];
#pragma unroll
        for (int i = 0; i < 2 * R; ++i) q1[i] = q1[i + 1];
        q1[2 * R] = from_arr(np1);
        // the slot of row y - R - 1 is free now: it takes row y + DEPTH (the
        // other lanes read it last in the previous iteration, before this
        // iteration's sync)
        if (y + F2_DEPTH < yb) {
            issue(y + F2_DEPTH, slot2);
            issue_img(y + F2_DEPTH, islot);
        }
        cp_commit();
        islot = (islot + 1 == F2_DEPTH) ? 0 : islot + 1;
        slot = (slot + 1 == RG::SLOTS) ? 0 : slot + 1;
        slotx = (slotx + 1 == RG::SLOTS) ? 0 : slotx + 1;
        slot2 = (slot2 + 1 == RG::SLOTS) ? 0 : slot2 + 1;
        l1 = (l1 + 1 == RG::Q1) ? 0 : l1 + 1;
        l2 = (l2 + 1 == RG::Q1) ? 0 : l2 + 1;
    }
    cp_wait<0>();
}

// ---------------------------------------------------------------------------
// Two-step tiles, variant 1: the same tile, rows and arithmetic as
// k_step2_interior, with the p_{n+1} rows kept only in shared lines (no
// register queue), so that the kernel fits in 128 registers and four blocks
// of four warps share an SM.  Per warp (float4 units):
//   row slots  NS = R + D + 1 slots; padded row r lives in slot (r - ya) mod NS:
//              p_n row r with its halo float4s [HL | 32 lanes | HR] (the
//              x-neighbours of the first step at row r, and the register
//              queue's new entry when row r - R is computed) and c2 row r (the
//              first step at row r, the second step at row r);
//   p_{n-1}    D lines, row r in line (r - ya) mod D;
//   p_{n+1}    NQ = 2R + 2 lines [garbage | 32 lanes | garbage], row r in line
//              (r - ya) mod NQ: the y- and x-neighbours of the second step;
//   inj        one line for a row's injected values / recorded receivers;
//   imaging    D slots of F2_ISIZE (snapshot row, accumulator row).
// D rows are in flight.  Every shared line a lane reads was written before
// the __syncwarp that opens the row iteration, or by the lane itself.
// ---------------------------------------------------------------------------
template <int R, bool IMG>
struct F2S {
    static constexpr int D = IMG ? 2 : 3;
    static constexpr int NS = R + D + 1;
    static constexpr int SLOT = 66, SPN = 0, SC2 = 34;
    static constexpr int NQ = 2 * R + 2;
    static constexpr int P1 = NS * SLOT;
    static constexpr int Q = P1 + D * 32;
    static constexpr int INJ = Q + NQ * F2_LINE;
    static constexpr int IR = INJ + F2_LINE;
    static constexpr int WARP = IR + (IMG ? D * F2_ISIZE : 0);  // float4 per warp
    static constexpr int SMEM = 4 * WARP * 16;
    // blocks per SM that the 228 KB of shared memory allow (1 KB reserved per block)
    static constexpr int BLOCKS = (228 * 1024) / (SMEM + 1024) >= 4 ? 4 : 3;
};

// x mod N for 0 <= x < 2N
template <int N>
__device__ __forceinline__ int wrapn(int x) {
    if constexpr ((N & (N - 1)) == 0) return x & (N - 1);
    else return x >= N ? x - N : x;
}

template <int R, int MODE, bool SNAP>
__global__ void __launch_bounds__(128, F2S<R, MODE == 1 && SNAP>::BLOCKS)
    k_step2s_interior(const __grid_constant__ StepParams P) {
    constexpr bool IMG = MODE == 1 && SNAP;
    using G = F2S<R, IMG>;
    constexpr int D = G::D, NS = G::NS, NQ = G::NQ;
    extern __shared__ float4 smem[];
    const int lane = threadIdx.x & 31;
    const int wid = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (wid >= P.nitems) return;
    float4* const wb = smem + (threadIdx.x >> 5) * G::WARP;
    float4* const slots = wb;
    float4* const p1r = wb + G::P1;
    float4* const q1l = wb + G::Q;
    float4* const inj = wb + G::INJ;
    float4* const iring = wb + G::IR;
    const WorkItem it = P.items[wid];
    const ShotDev& S = P.shots[it.shot];
    const int pitch = S.pitch, dn = S.dn;
    const int x0 = it.tile, xl = x0 - 4 + 4 * lane;
    const float* PN = S.pf[P.rp] + xl;    // p_n
    const float* PM = S.pf[P.rp1] + xl;   // p_{n-1}
    float* O1 = S.pf[P.wo] + xl;          // p_{n+1}
    float* O2 = S.pf[P.wo2] + xl;         // p_{n+2}
    const float* C2 = S.c2 + xl;
    // lanes 0 and 31 also fetch the halo float4 beyond the warp's columns
    const bool has_h = (lane == 0) || (lane == 31);
    const int hidx = (lane == 0) ? 0 : 33, hoff = (lane == 0) ? -4 : 4;
    // lanes 1..30 store their elements [lo, hi): the interior columns [sl, sr)
    const int lo = S.off + S.sl - xl, hi = S.off + S.sr - xl;
    const bool mine = lane >= 1 && lane <= 30;
    const bool full = mine && lo <= 0 && hi >= 4, part = mine && !full && lo < 4 && hi > 0;
    const int y0 = it.y0, y1 = it.y1, ya = y0 - R, yb = y1 + R + 1;

    auto issue_pn = [&](int r, int s) {  // p_n row r (with halos) into slot s
        float4* d = slots + s * G::SLOT + G::SPN;
        const float* src = PN + (size_t)r * pitch;
        cp16(d + 1 + lane, src);
        if (has_h) cp16(d + hidx, src + hoff);
    };
    auto issue_row = [&](int r, int s, int l) {  // p_{n-1} row r into line l, c2 row r into slot s
        cp16(p1r + l * 32 + lane, PM + (size_t)r * pitch);
        cp16(slots + s * G::SLOT + G::SC2 + lane, C2 + (size_t)r * pitch);
    };
    auto issue_img = [&](int y, int islot) {
        if (!IMG || y < y0 || y >= y1) return;
        float4* isl = iring + islot * F2_ISIZE;
        const int yrow = y - dn;
        const size_t fo = (size_t)P.snap * (size_t)S.snap_stride + (size_t)yrow * pitch + xl;
        if (P.snap_form == 0) {
            cp16(isl + F2_IF + lane, reinterpret_cast<const float*>(S.snaps) + fo);
        } else {
            cp8(reinterpret_cast<uint2*>(isl + F2_IF) + lane, reinterpret_cast<const unsigned short*>(S.snaps) + fo);
            cp4(reinterpret_cast<float*>(isl + F2_IS) + lane,
                S.sscale + ((size_t)P.snap * S.ny + yrow) * (S.ntiles + 2) + (xl >> 7));
        }
        const size_t ko = (size_t)yrow * pitch + xl;
        if (P.grad_form == 0) {
            cp16(isl + F2_IK + lane, S.k32 + ko);
        } else {
            cp16(isl + F2_IK + 2 * lane, S.k64 + ko);
            cp16(isl + F2_IK + 2 * lane + 1, S.k64 + ko + 2);
        }
    };
    // p_n rows ya .. ya+R-1 (x-neighbours only), then D groups of row ya+j
#pragma unroll
    for (int i = 0; i < R; ++i) issue_pn(ya + i, i);
    cp_commit();
#pragma unroll
    for (int j = 0; j < D; ++j) {
        issue_pn(ya + j + R, j + R);
        issue_row(ya + j, j, j);
        issue_img(ya + j, j);
        cp_commit();
    }
    // qn: p_n rows y-R-1 .. y+R (the last one from the slot in the row iteration)
    float4 qn[2 * R + 2];
#pragma unroll
    for (int i = 0; i < 2 * R + 1; ++i) qn[i] = ldg4(PN + (size_t)(ya - R - 1 + i) * pitch);

    // source cursors: first step from the list start, second step from row y0
    int si1 = it.s0, si2 = it.s0, ri1 = it.r0, ri2 = it.r0;
    while (si2 < it.s1 && P.srcs[si2].row < y0) ++si2;
    int srow1 = (si1 < it.s1) ? P.srcs[si1].row : INT_MAX, srow2 = (si2 < it.s1) ? P.srcs[si2].row : INT_MAX;
    int rrow1 = (ri1 < it.r1) ? P.recs[ri1].row : INT_MAX, rrow2 = rrow1;
    float2 cp[R + 1];
#pragma unroll
    for (int i = 0; i <= R; ++i) cp[i] = make_float2(P.c2[i], P.c2[i]);

    // slot of row y (s0), of row y+R (sR), of row y-R-1 = row y+D (s2), of row
    // y-1 = row y+D+R (sp); p_{n-1} line of row y (l1); p_{n+1} line of row y (lq)
    int s0 = 0, sR = R, s2 = D, sp = NS - 1, l1 = 0, lq = 0;
    for (int y = ya; y < yb; ++y) {
        cp_wait<D - 1>();
        __syncwarp();
        const float4* st = slots + s0 * G::SLOT;
        qn[2 * R + 1] = slots[sR * G::SLOT + G::SPN + 1 + lane];
        const float4 pm1 = p1r[l1 * 32 + lane];
        // first step, row y: p_{n+1} = -p_{n-1} + 2p_n + (d2x + d2y + source)*c2
        float np1[4] = {0.f, 0.f, 0.f, 0.f};
        {
            float sv[4] = {0.f, 0.f, 0.f, 0.f};
            if (srow1 == y) to_arr(gather_sources(P, S, y, x0 - 4, P.t, si1, it.s1, srow1, inj, lane), sv);
            if (y >= dn)
                interior_update2<R>(qn + 1, st[G::SPN + lane], st[G::SPN + 2 + lane], pm1, st[G::SC2 + lane], sv, cp,
                                    np1);
        }
        float4* const lnw = q1l + lq * F2_LINE;
        lnw[1 + lane] = from_arr(np1);
        // second step, row y - R - 1, from the p_{n+1} lines of rows y-2R-1 .. y-1
        // (lines lq+1 .. lq+2R+1 mod NQ)
        const int y2 = y - R - 1;
        if (y2 >= y0) {
            const int b = wrapn<NQ>(lq + 1);
            const float4* lc = q1l + wrapn<NQ>(b + R) * F2_LINE;
            float sv[4] = {0.f, 0.f, 0.f, 0.f};
            if (srow2 == y2) to_arr(gather_sources(P, S, y2, x0 - 4, P.t + 1, si2, it.s1, srow2, inj, lane), sv);
            float np2[4];
            interior_update2f<R>(
                [&](int j) { return q1l[wrapn<NQ>(b + j) * F2_LINE + 1 + lane]; }, lc[lane], lc[lane + 2], qn[0],
                slots[s2 * G::SLOT + G::SC2 + lane], sv, cp, np2);
            if (full) {
                st4(O2 + (size_t)y2 * pitch, from_arr(np2));
            } else if (part) {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (e >= lo && e < hi) O2[(size_t)y2 * pitch + e] = np2[e];
            }
            if (MODE == 0 && P.record && rrow2 == y2) {
                inj[1 + lane] = from_arr(np2);  // the injection line is free again
                __syncwarp();
                record_row_par(P, S, y2, x0 - 4, P.t + 1, ri2, it.r1, rrow2, inj, lane);
            }
        }
        if (y >= y0 && y < y1) {
            if (full) {
                st4(O1 + (size_t)y * pitch, from_arr(np1));
            } else if (part) {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (e >= lo && e < hi) O1[(size_t)y * pitch + e] = np1[e];
            }
            if (MODE == 0 && P.record && rrow1 == y) {
                __syncwarp();  // np1 of every lane is in its p_{n+1} line
                record_row_par(P, S, y, x0 - 4, P.t, ri1, it.r1, rrow1, lnw, lane);
            }
            if (SNAP && (full || part))
                snap_or_image<MODE>(P, S, y - dn, xl, lo, hi, full, np1, pm1, iring + l1 * F2_ISIZE, lane);
        }
#pragma unroll
        for (int i = 0; i < 2 * R + 1; ++i) qn[i] = qn[i + 1];
        // row y + D: p_n row y+D+R into the slot of row y-1 (its p_n was last
        // read in the previous iteration), p_{n-1} and c2 into the line and slot
        // whose rows this lane has just used
        if (y + D < yb) {
            issue_pn(y + D + R, sp);
            issue_row(y + D, s2, l1);
            issue_img(y + D, l1);  // the imaging slot of row y, used above
        }
        cp_commit();
        s0 = wrapn<NS>(s0 + 1);
        sR = wrapn<NS>(sR + 1);
        s2 = wrapn<NS>(s2 + 1);
        sp = wrapn<NS>(sp + 1);
        l1 = wrapn<D>(l1 + 1);
        lq = wrapn<NQ>(lq + 1);
    }
    cp_wait<0>();
}

// Bottom pad rows, interior columns: the boundary list after its nstrip
// side-strip items.  Runs on its own stream, concurrently with
// k_step_interior and k_step_strip.
constexpr int BND_SMEM = 4 * BOT_DEPTH * SB_SIZE * 16;

// One single step of a small wave in one launch: blocks [0, bm) take the
// interior list, [bm, bm + bs) the side strips, the rest the bottom tiles --
// the work of k_step_interior, k_step_strip and k_step_bottom, which touch
// disjoint cells and read only the step's inputs.  A small wave's step is
// latency-bound; one launch instead of three on three streams (forked and
// joined around every step) takes the fork, the join and two launches out
// of it.
template <int R, int MODE, bool SNAP, int K>
__global__ void __launch_bounds__(128, 3)
    k_step_fused(const __grid_constant__ StepParams Pm, const __grid_constant__ StepParams Pb, int bm, int bs) {
    extern __shared__ float4 smem[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int b = blockIdx.x;
    if (b < bm) {
        interior_rows<R, MODE, SNAP>(Pm, b * 4 + w, w, smem);
        return;
    }
    b -= bm;
    if (b < bs) {
        const int wid = b * 4 + w;
        if (wid >= Pb.nstrip) return;
        float* sw = reinterpret_cast<float*>(smem) + w * StripLayout<R, K>::WARP;
        const WorkItem it = Pb.items[wid];
        if (it.kind == 3) strip_rows<R, MODE, K, true>(Pb, it, sw, lane);
        else strip_rows<R, MODE, K, false>(Pb, it, sw, lane);
        return;
    }
    b -= bs;
    const int wid = Pb.nstrip + b * 4 + w;
    if (wid >= Pb.nitems) return;
    bottom_rows<R, MODE>(Pb, Pb.items[wid], smem + w * (BOT_DEPTH * SB_SIZE), lane);
}

template <int R, int MODE, bool SNAP, int K>
constexpr int fused_smem() {
    constexpr int a = (MODE == 1 && SNAP) ? IN_SMEM_IMG : IN_SMEM, b = strip_smem<R, K>(), c = BND_SMEM;
    return a > b ? (a > c ? a : c) : (b > c ? b : c);
}

template <int R, int MODE>
__global__ void __launch_bounds__(128, 3) k_step_bottom(const __grid_constant__ StepParams P) {
    extern __shared__ float4 smem[];
    const int lane = threadIdx.x & 31;
    const int wid = P.nstrip + blockIdx.x * 4 + (threadIdx.x >> 5);
    if (wid >= P.nitems) return;
    float4* ring = smem + (threadIdx.x >> 5) * (BOT_DEPTH * SB_SIZE);
    const WorkItem it = P.items[wid];
    bottom_rows<R, MODE>(P, it, ring, lane);
}

// Opt the step kernels into the dynamic shared memory they use (above the
// 48 KB default) and into the largest shared-memory carveout: the step
// kernels share SMs, and with it every one of them reaches its
// register-limited occupancy.
template <typename KernelT>
cudaError_t kernel_smem(KernelT* k, int bytes) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    return e;
}

template <int R, int MODE>
cudaError_t configure_variant() {
    cudaError_t e = kernel_smem(k_step_interior<R, MODE, false>, IN_SMEM);
    if (e == cudaSuccess) e = kernel_smem(k_step_interior<R, MODE, true>, MODE == 1 ? IN_SMEM_IMG : IN_SMEM);
    if (e == cudaSuccess) e = kernel_smem(k_step_bottom<R, MODE>, BND_SMEM);
    if (e == cudaSuccess) e = kernel_smem(k_step_strip<R, MODE, 1>, strip_smem<R, 1>());
    if (e == cudaSuccess) e = kernel_smem(k_step_strip<R, MODE, 2>, strip_smem<R, 2>());
    if (e == cudaSuccess) e = kernel_smem(k_step2_interior<R, MODE, false>, F2Ring<R>::SMEM);
    if (e == cudaSuccess) e = kernel_smem(k_step2_interior<R, MODE, true>, F2Ring<R, MODE == 1>::SMEM);
    if (e == cudaSuccess) e = kernel_smem(k_step2s_interior<R, MODE, false>, F2S<R, false>::SMEM);
    if (e == cudaSuccess) e = kernel_smem(k_step2s_interior<R, MODE, true>, F2S<R, MODE == 1>::SMEM);
    if (e == cudaSuccess) e = kernel_smem(k_step_fused<R, MODE, false, 1>, fused_smem<R, MODE, false, 1>());
    if (e == cudaSuccess) e = kernel_smem(k_step_fused<R, MODE, true, 1>, fused_smem<R, MODE, true, 1>());
    if (e == cudaSuccess) e = kernel_smem(k_step_fused<R, MODE, false, 2>, fused_smem<R, MODE, false, 2>());
    if (e == cudaSuccess) e = kernel_smem(k_step_fused<R, MODE, true, 2>, fused_smem<R, MODE, true, 2>());
    return e;
}

cudaError_t configure_step_kernels() {
    cudaError_t e = configure_variant<3, 0>();
    if (e == cudaSuccess) e = configure_variant<3, 1>();
    if (e == cudaSuccess) e = configure_variant<4, 0>();
    if (e == cudaSuccess) e = configure_variant<4, 1>();
    return e;
}

template <int R, int MODE>
void launch_variant(int kstrip, const StepParams& pm, const StepParams& pb, cudaStream_t sm, cudaStream_t sb,
                    cudaStream_t ss) {
    const int bm = (pm.nitems + 3) / 4, bs = (pb.nstrip + 3) / 4, bb = (pb.nitems - pb.nstrip + 3) / 4;
    if (bs) {
        if (kstrip == 1) k_step_strip<R, MODE, 1><<<bs, 128, strip_smem<R, 1>(), ss>>>(pb);
        else k_step_strip<R, MODE, 2><<<bs, 128, strip_smem<R, 2>(), ss>>>(pb);
    }
    if (bb) k_step_bottom<R, MODE><<<bb, 128, BND_SMEM, sb>>>(pb);
    if (bm) {
        if (pm.snap >= 0)
            k_step_interior<R, MODE, true><<<bm, 128, MODE == 1 ? IN_SMEM_IMG : IN_SMEM, sm>>>(pm);
        else
            k_step_interior<R, MODE, false><<<bm, 128, IN_SMEM, sm>>>(pm);
    }
}

// Interior kernel on stream sm, bottom tiles on sb, side strips (model and
// bottom rows) on ss; the caller orders the streams around each time step.
// kstrip = columns per lane of the strip kernel (ceil(strip width / 32)).
cudaError_t launch_step(int acc, int mode, int kstrip, const StepParams& pm, const StepParams& pb, cudaStream_t sm,
                        cudaStream_t sb, cudaStream_t ss) {
    if (kstrip != 1 && kstrip != 2) return cudaErrorInvalidValue;
    if (acc == 3) {
        if (mode == 0) launch_variant<3, 0>(kstrip, pm, pb, sm, sb, ss);
        else launch_variant<3, 1>(kstrip, pm, pb, sm, sb, ss);
    } else if (acc == 4) {
        if (mode == 0) launch_variant<4, 0>(kstrip, pm, pb, sm, sb, ss);
        else launch_variant<4, 1>(kstrip, pm, pb, sm, sb, ss);
    } else {
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <int R, int MODE>
void launch_fused_variant(int kstrip, const StepParams& pm, const StepParams& pb, cudaStream_t st) {
    const int bm = (pm.nitems + 3) / 4, bs = (pb.nstrip + 3) / 4, bb = (pb.nitems - pb.nstrip + 3) / 4;
    const int nb = bm + bs + bb;
    if (!nb) return;
    if (kstrip == 1) {
        if (pm.snap >= 0) k_step_fused<R, MODE, true, 1><<<nb, 128, fused_smem<R, MODE, true, 1>(), st>>>(pm, pb, bm, bs);
        else k_step_fused<R, MODE, false, 1><<<nb, 128, fused_smem<R, MODE, false, 1>(), st>>>(pm, pb, bm, bs);
    } else {
        if (pm.snap >= 0) k_step_fused<R, MODE, true, 2><<<nb, 128, fused_smem<R, MODE, true, 2>(), st>>>(pm, pb, bm, bs);
        else k_step_fused<R, MODE, false, 2><<<nb, 128, fused_smem<R, MODE, false, 2>(), st>>>(pm, pb, bm, bs);
    }
}

// One single step in one launch (k_step_fused) on stream st.
cudaError_t launch_step_fused(int acc, int mode, int kstrip, const StepParams& pm, const StepParams& pb,
                              cudaStream_t st) {
    if (kstrip != 1 && kstrip != 2) return cudaErrorInvalidValue;
    if (acc == 3) {
        if (mode == 0) launch_fused_variant<3, 0>(kstrip, pm, pb, st);
        else launch_fused_variant<3, 1>(kstrip, pm, pb, st);
    } else if (acc == 4) {
        if (mode == 0) launch_fused_variant<4, 0>(kstrip, pm, pb, st);
        else launch_fused_variant<4, 1>(kstrip, pm, pb, st);
    } else {
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <int R, int MODE>
void launch_step2_variant(int var, const StepParams& pf, int nb, cudaStream_t st) {
    if (var == 1) {
        if (pf.snap >= 0) k_step2s_interior<R, MODE, true><<<nb, 128, F2S<R, MODE == 1>::SMEM, st>>>(pf);
        else k_step2s_interior<R, MODE, false><<<nb, 128, F2S<R, false>::SMEM, st>>>(pf);
        return;
    }
    if (pf.snap >= 0) k_step2_interior<R, MODE, true><<<nb, 128, F2Ring<R, MODE == 1>::SMEM, st>>>(pf);
    else k_step2_interior<R, MODE, false><<<nb, 128, F2Ring<R>::SMEM, st>>>(pf);
}

// Two-step interior tiles (kind 4) of list pf on stream st; pf.snap >= 0:
// the first step stores that snapshot block / images with it.  var selects
// the kernel: 0 = k_step2_interior (register queues, three blocks per SM),
// 1 = k_step2s_interior (p_{n+1} rows in shared memory, up to four blocks
// per SM); both compute the same cells with the same arithmetic.
cudaError_t launch_step2(int acc, int mode, int var, const StepParams& pf, cudaStream_t st) {
    const int nb = (pf.nitems + 3) / 4;
    if (!nb) return cudaSuccess;
    if (mode == 0 && pf.snap >= 0 && pf.snap_form != 0) return cudaErrorInvalidValue;  // FP32 snapshots only
    if (var != 0 && var != 1) return cudaErrorInvalidValue;
    if (acc == 3) {
        if (mode == 0) launch_step2_variant<3, 0>(var, pf, nb, st);
        else launch_step2_variant<3, 1>(var, pf, nb, st);
    } else if (acc == 4) {
        if (mode == 0) launch_step2_variant<4, 0>(var, pf, nb, st);
        else launch_step2_variant<4, 1>(var, pf, nb, st);
    } else {
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace fwi
