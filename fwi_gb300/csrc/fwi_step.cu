// FWI time-step kernels for sm_103a.
//
// One launch of k_step_main plus one of k_step_bottom advance every shot of a
// wave by one time step of the reference solver (solver_acoustic_SS.f90:313-586):
//
//   k_step_main    model rows dn..dn+ny-1: interior update with source
//                  injection (:319-330, :433-434), left/right CPML strips
//                  (pml_matrices_x, solver_PML_matrices.f90:1-40), snapshot
//                  store (:438-454) or imaging condition (:457-473),
//                  receiver recording (:551-555);
//   k_step_bottom  bottom pad rows: bottom CPML strip (pml_matrices_y
//                  :42-81) and the two bottom corners in two stages
//                  (pml_matrices_xycorner :83-112, solver_acoustic_SS.f90:395-411).
//
// The top pad rows are never written: with the free surface they stay
// exactly zero for the whole run (solver_acoustic_SS.f90:416-429, :477-479).
//
// Every warp owns a 128-column tile (4 columns per lane, float4) and marches
// down a band of rows; the y-stencil comes from a register queue of 2R+1
// rows, the x-stencil from warp shuffles of the current row plus one halo
// float4 at each end of the tile.  The wavefield is ping-ponged between two
// buffers: p_3 overwrites p_1 in place (each cell reads its own p_1 only).
// The CPML memory variables are updated in place: the strip-local
// derivative of phi only reads phi values of the same warp, loaded before
// they are overwritten.
//
// This file is compiled with --fmad=false: every a*b+c below is a rounded
// multiply followed by a rounded add, in the order the Fortran source writes
// the expression, so results are bit-identical to the reference arithmetic.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <climits>

#include "fwi_internal.cuh"

namespace fwi {

namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }

__device__ __forceinline__ void to_arr(float4 v, float* a) { a[0] = v.x; a[1] = v.y; a[2] = v.z; a[3] = v.w; }
__device__ __forceinline__ float4 from_arr(const float* a) { return make_float4(a[0], a[1], a[2], a[3]); }
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

// space_deriv2x / space_derivx at this lane's columns (solver_space_derivs.f90:11-16, :70-82)
template <int R>
__device__ __forceinline__ void xderivs(const float* w, const StepParams& P, float* d2, float* d1) {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        float s2 = 0.f, s1 = 0.f;
#pragma unroll
        for (int i = 0; i <= R; ++i) {
            s2 = s2 + P.c2[i] * (w[4 + e + i] + w[4 + e - i]);
            s1 = s1 + (w[4 + e + i] - w[4 + e - i]) * P.c1[i];
        }
        d2[e] = s2;
        d1[e] = s1;
    }
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

// Second derivatives only (interior cells need no first derivative).
template <int R>
__device__ __forceinline__ void xderiv2(const float* w, const StepParams& P, float* d2) {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        float s2 = 0.f;
#pragma unroll
        for (int i = 0; i <= R; ++i) s2 = s2 + P.c2[i] * (w[4 + e + i] + w[4 + e - i]);
        d2[e] = s2;
    }
}
template <int R>
__device__ __forceinline__ void yderiv2(const float4* q, const StepParams& P, float* d2) {
    float a[2 * R + 1][4];
#pragma unroll
    for (int i = 0; i <= 2 * R; ++i) to_arr(q[i], a[i]);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        float s2 = 0.f;
#pragma unroll
        for (int i = 0; i <= R; ++i) s2 = s2 + (a[R + i][e] + a[R - i][e]) * P.c2[i];
        d2[e] = s2;
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

// Fetch element `col` (physical, inside this tile) of a per-lane 4-array.
__device__ __forceinline__ float fetch(const float* a, int col_in_tile) {
    const int ln = col_in_tile >> 2, el = col_in_tile & 3;
    return __shfl_sync(FULL, sel(a, el), ln);
}

// Grid-edge clamp of the x derivatives: columns < R copy column R, columns
// > nxt-1-R copy column nxt-1-R (solver_space_derivs.f90:18-23, :84-94).
template <int R>
__device__ __forceinline__ void xclamp(const ShotDev& S, int x0, int c0, bool first, bool last, float* d2, float* d1) {
    if (first) {
        const int ct = S.off + R - x0;
        const float v2 = fetch(d2, ct), v1 = fetch(d1, ct);
#pragma unroll
        for (int e = 0; e < 4; ++e)
            if (c0 + e < R) { d2[e] = v2; d1[e] = v1; }
    }
    if (last) {
        const int ct = S.off + S.nxt - 1 - R - x0;
        const float v2 = fetch(d2, ct), v1 = fetch(d1, ct);
#pragma unroll
        for (int e = 0; e < 4; ++e)
            if (c0 + e > S.nxt - 1 - R) { d2[e] = v2; d1[e] = v1; }
    }
}

// Strip-local x derivative of the old x-direction phi with the strip-edge
// clamp (pml_matrices_x / _xycorner call space_derivx on the dn-wide strip
// array, solver_PML_matrices.f90:15, :97).  Valid for columns of the side
// strips / corners only.
template <int R>
__device__ __forceinline__ void phi_xderiv(const ShotDev& S, const StepParams& P, float4 ph, int lane, int x0, int c0,
                                           bool first, bool last, float* dph) {
    float w[12];
    window(ph, ph, ph, lane, w);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        float s1 = 0.f;
#pragma unroll
        for (int i = 0; i <= R; ++i) s1 = s1 + (w[4 + e + i] - w[4 + e - i]) * P.c1[i];
        dph[e] = s1;
    }
    const int dn = S.dn, nx = S.nx;
    if (first) {
        const float lo = fetch(dph, S.off + R - x0), hi = fetch(dph, S.off + dn - 1 - R - x0);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int c = c0 + e;
            if (c < dn) {
                if (c < R) dph[e] = lo;
                else if (c > dn - 1 - R) dph[e] = hi;
            }
        }
    }
    if (last) {
        const int base = dn + nx;
        const float lo = fetch(dph, S.off + base + R - x0), hi = fetch(dph, S.off + base + dn - 1 - R - x0);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int il = c0 + e - base;
            if (il >= 0) {
                if (il < R) dph[e] = lo;
                else if (il > dn - 1 - R) dph[e] = hi;
            }
        }
    }
}

// Snapshot store (forward) of the interior cells of one row:
// Fields(j, snap*nx+i) = (p_3 - p_1)*0.5/dt   (solver_acoustic_SS.f90:447)
__device__ __forceinline__ void store_snapshot(const StepParams& P, const ShotDev& S, int yrow, int lane, int x0,
                                               int xl, int c0, const float* p3, const float* pm1, int tile) {
    const int dn = S.dn, nx = S.nx;
    float v[4];
    bool in[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int c = c0 + e;
        in[e] = (c >= dn) && (c < dn + nx);
        v[e] = in[e] ? ((p3[e] - pm1[e]) * 0.5f) / P.dt : 0.f;
    }
    const size_t base = (size_t)P.snap * (size_t)S.snap_stride + (size_t)yrow * S.pitch + xl;
    if (P.snap_form == 0) {
        float* F = reinterpret_cast<float*>(S.snaps) + base;
        if (in[0] && in[3]) {
            st4(F, from_arr(v));
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (in[e]) F[e] = v[e];
        }
        return;
    }
    // 16-bit forms: power-of-two scale per 128-column row segment so that the
    // largest magnitude maps below 2^14 (exact scaling, no extra rounding).
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
    if (in[0] && in[3]) {
        uint2 pk;
        pk.x = (unsigned)h[0] | ((unsigned)h[1] << 16);
        pk.y = (unsigned)h[2] | ((unsigned)h[3] << 16);
        *reinterpret_cast<uint2*>(F) = pk;
    } else {
#pragma unroll
        for (int e = 0; e < 4; ++e)
            if (in[e]) F[e] = h[e];
    }
    if (lane == 0) {
        S.sscale[((size_t)P.snap * S.ny + yrow) * S.ntiles + tile] = ldexpf(1.f, -sh);
    }
}

// Imaging condition (adjoint): kernel += -0.5*(p_3-p_1)*Fields(snap)*store_snap
// (solver_acoustic_SS.f90:465-466)
__device__ __forceinline__ void image_row(const StepParams& P, const ShotDev& S, int yrow, int xl, int c0,
                                          const float* p3, const float* pm1, int tile) {
    const int dn = S.dn, nx = S.nx;
    const size_t base = (size_t)P.snap * (size_t)S.snap_stride + (size_t)yrow * S.pitch + xl;
    float F[4];
    if (P.snap_form == 0) {
        to_arr(ldg4(reinterpret_cast<const float*>(S.snaps) + base), F);
    } else {
        const uint2 pk = __ldg(reinterpret_cast<const uint2*>(reinterpret_cast<const unsigned short*>(S.snaps) + base));
        const unsigned short h[4] = {(unsigned short)(pk.x & 0xffffu), (unsigned short)(pk.x >> 16),
                                     (unsigned short)(pk.y & 0xffffu), (unsigned short)(pk.y >> 16)};
        const float sc = __ldg(S.sscale + ((size_t)P.snap * S.ny + yrow) * S.ntiles + tile);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            float f;
            if (P.snap_form == 1) f = __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(&h[e]));
            else f = __half2float(*reinterpret_cast<const __half*>(&h[e]));
            F[e] = f * sc;
        }
    }
    float k2[4];
    bool in[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int c = c0 + e;
        in[e] = (c >= dn) && (c < dn + nx);
        k2[e] = -(((0.5f * (p3[e] - pm1[e])) * F[e]) * P.ss);
    }
    const size_t ko = (size_t)yrow * S.pitch + xl;
    if (P.grad_form == 0) {
        float* K = S.k32 + ko;
        if (in[0] && in[3]) {
            float4 k = ld4(K);
            k.x = k.x + k2[0]; k.y = k.y + k2[1]; k.z = k.z + k2[2]; k.w = k.w + k2[3];
            st4(K, k);
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (in[e]) K[e] = K[e] + k2[e];
        }
    } else {
        double* K = S.k64 + ko;
        if (in[0] && in[3]) {
            double2* K2 = reinterpret_cast<double2*>(K);
            double2 a = K2[0], b = K2[1];
            a.x += (double)k2[0]; a.y += (double)k2[1]; b.x += (double)k2[2]; b.y += (double)k2[3];
            K2[0] = a;
            K2[1] = b;
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (in[e]) K[e] += (double)k2[e];
        }
    }
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

// One prefetch stage of the main kernel (float4 slots): p(y+R), p_1(y),
// c2(y), x-phi(y), x-chi(y) per lane, plus the two halo float4 of p(y).
constexpr int ST_P = 0, ST_P1 = 32, ST_C2 = 64, ST_PH = 96, ST_CH = 128, ST_HL = 160, ST_HR = 161, ST_SIZE = 162;
constexpr int MAIN_DEPTH = 4;  // rows in flight per warp
constexpr int MAIN_SMEM = 4 * MAIN_DEPTH * ST_SIZE * 16;  // bytes per 4-warp block

// Model rows of the first and last tile of a shot: interior cells plus the
// left/right CPML strips, with the grid-edge clamps of the x derivatives.
template <int R, int MODE>
__device__ __forceinline__ void edge_rows(const StepParams& P, const WorkItem& it, float4* ring, int lane) {
    const ShotDev& S = P.shots[it.shot];
    const int pitch = S.pitch, dn = S.dn, nx = S.nx, nxt = S.nxt;
    const int x0 = it.tile * TILE, xl = x0 + 4 * lane, c0 = xl - S.off;
    const bool first = it.tile == 0, last = it.tile == S.ntiles - 1, edge = first || last;
    const float* PC = P.parity ? S.pa : S.pb;  // p
    float* P1 = P.parity ? S.pb : S.pa;        // p_1, overwritten with p_3
    bool lane_strip = false;
    if (edge) lane_strip = (c0 < dn) || (c0 + 3 >= dn + nx);
    const bool has_hl = (lane == 0) && (x0 > 0), has_hr = (lane == 31) && (x0 + TILE < pitch);

    auto issue = [&](int y, int slot) {
        float4* st = ring + slot * ST_SIZE;
        const size_t ro = (size_t)y * pitch + xl;
        cp16(st + ST_P + lane, PC + (size_t)(y + R) * pitch + xl);
        cp16(st + ST_P1 + lane, P1 + ro);
        cp16(st + ST_C2 + lane, S.c2 + ro);
        if (lane_strip) {
            cp16(st + ST_PH + lane, S.phx + ro);
            cp16(st + ST_CH + lane, S.chx + ro);
        }
        if (has_hl) cp16(st + ST_HL, PC + (size_t)y * pitch + x0 - 4);
        if (has_hr) cp16(st + ST_HR, PC + (size_t)y * pitch + x0 + TILE);
    };

#pragma unroll
    for (int i = 0; i < MAIN_DEPTH; ++i) {
        if (it.y0 + i < it.y1) issue(it.y0 + i, i);
        cp_commit();
    }
    float4 q[2 * R + 1];
#pragma unroll
    for (int i = 0; i < 2 * R; ++i) q[i] = ldg4(PC + (size_t)(it.y0 - R + i) * pitch + xl);

    int si = it.s0, ri = it.r0;
    int srow = (si < it.s1) ? P.srcs[si].row : INT_MAX;
    int rrow = (ri < it.r1) ? P.recs[ri].row : INT_MAX;

    int slot = 0;
    for (int y = it.y0; y < it.y1; ++y) {
        cp_wait<MAIN_DEPTH - 1>();
        const float4* st = ring + slot * ST_SIZE;
        const size_t ro = (size_t)y * pitch + xl;
        q[2 * R] = st[ST_P + lane];
        float pm1[4], cc[4], pc[4];
        to_arr(st[ST_P1 + lane], pm1);
        to_arr(st[ST_C2 + lane], cc);
        to_arr(q[R], pc);
        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 hl = has_hl ? st[ST_HL] : z4, hr = has_hr ? st[ST_HR] : z4;
        float ph[4] = {0.f, 0.f, 0.f, 0.f}, ch[4] = {0.f, 0.f, 0.f, 0.f};
        if (lane_strip) {
            to_arr(st[ST_PH + lane], ph);
            to_arr(st[ST_CH + lane], ch);
        }
        float w[12];
        window(q[R], hl, hr, lane, w);
        float d2x[4], dx[4], d2y[4];
        xderivs<R>(w, P, d2x, dx);
        yderiv2<R>(q, P, d2y);

        // source injection: source(nys,nxs) = S(k-1,j), interior cells only
        float sv[4] = {0.f, 0.f, 0.f, 0.f};
        while (srow == y) {
            const SrcEnt s = P.srcs[si];
            if ((s.col >> 2) == (xl >> 2)) {
                const float val = __ldg(S.srcv + (size_t)s.vidx * S.nt + P.t);
                const int el = s.col & 3;
                sv[0] = el == 0 ? val : sv[0];
                sv[1] = el == 1 ? val : sv[1];
                sv[2] = el == 2 ? val : sv[2];
                sv[3] = el == 3 ? val : sv[3];
            }
            ++si;
            srow = (si < it.s1) ? P.srcs[si].row : INT_MAX;
        }

        float p3[4];
        if (!edge) {
#pragma unroll
            for (int e = 0; e < 4; ++e)
                p3[e] = ((-pm1[e]) + 2.f * pc[e]) + (((d2x[e] + d2y[e]) + sv[e]) * cc[e]);
        } else {
            xclamp<R>(S, x0, c0, first, last, d2x, dx);
            float dph[4];
            phi_xderiv<R>(S, P, from_arr(ph), lane, x0, c0, first, last, dph);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int c = c0 + e;
                if (c < 0 || c >= nxt) {
                    p3[e] = 0.f;
                } else if (c >= dn && c < dn + nx) {
                    p3[e] = ((-pm1[e]) + 2.f * pc[e]) + (((d2x[e] + d2y[e]) + sv[e]) * cc[e]);
                } else {
                    // xl strip: factor(dn-i+1); xr strip: factor(i)  (solver_PML_matrices.f90:296-312)
                    const int fi = (c < dn) ? (dn - 1 - c) : (c - dn - nx);
                    const float A = __ldg(P.fA + fi), B = __ldg(P.fB + fi);
                    const float phn = A * ph[e] + B * dx[e];
                    const float chn = A * ch[e] + B * (d2x[e] + dph[e]);
                    const float prop = dph[e] + chn;
                    ph[e] = phn;
                    ch[e] = chn;
                    p3[e] = ((-pm1[e]) + 2.f * pc[e]) + cc[e] * ((d2x[e] + d2y[e]) + prop);
                }
            }
            if (lane_strip) {
                st4(S.phx + ro, from_arr(ph));
                st4(S.chx + ro, from_arr(ch));
            }
        }

        if (MODE == 0 && P.snap >= 0) store_snapshot(P, S, y - dn, lane, x0, xl, c0, p3, pm1, it.tile);
        if (MODE == 1 && P.snap >= 0) image_row(P, S, y - dn, xl, c0, p3, pm1, it.tile);
        st4(P1 + ro, from_arr(p3));
        if (MODE == 0 && P.record) record_row(P, S, y, xl, ri, it.r1, rrow, p3);

#pragma unroll
        for (int i = 0; i < 2 * R; ++i) q[i] = q[i + 1];
        // refill this slot (its values are consumed above) with row y + depth
        if (y + MAIN_DEPTH < it.y1) issue(y + MAIN_DEPTH, slot);
        cp_commit();
        slot = (slot + 1 == MAIN_DEPTH) ? 0 : slot + 1;
    }
    cp_wait<0>();
}

// One prefetch stage of the bottom kernel: p(y+R), p_1(y), c2(y), y-phi(y),
// y-chi(y), x-phi(y), x-chi(y), the y-phi row the derivative queue needs
// next (jl+1+R), and the halo float4 of p(y).
constexpr int SB_P = 0, SB_P1 = 32, SB_C2 = 64, SB_PY = 96, SB_CY = 128, SB_PX = 160, SB_CX = 192, SB_FA = 224,
              SB_HL = 256, SB_HR = 257, SB_SIZE = 258;
constexpr int BOT_DEPTH = 3;
constexpr int BOT_SMEM = 4 * BOT_DEPTH * SB_SIZE * 16;

// Bottom pad rows [it.y0, it.y1) of one tile: bottom strip and bottom
// corners.  The y-direction phi is ping-ponged between two buffers (old read
// from one, new written to the other), so the strip-local derivative of the
// old phi can be taken in any band of the bottom pad.
template <int R, int MODE>
__device__ __forceinline__ void bottom_rows(const StepParams& P, const WorkItem& it, float4* ring, int lane) {
    const ShotDev& S = P.shots[it.shot];
    const int pitch = S.pitch, dn = S.dn, nx = S.nx, nxt = S.nxt, nyt = S.nyt;
    const int x0 = it.tile * TILE, xl = x0 + 4 * lane, c0 = xl - S.off;
    const bool first = it.tile == 0, last = it.tile == S.ntiles - 1, edge = first || last;
    const float* PC = P.parity ? S.pa : S.pb;
    float* P1 = P.parity ? S.pb : S.pa;
    const float* PHO = P.parity ? S.phy2 : S.phy;  // old y-phi
    float* PHN = P.parity ? S.phy : S.phy2;        // new y-phi
    const int yb0 = nyt - dn;
    const int j0 = it.y0 - yb0, j1 = it.y1 - yb0;
    const int jA = max(j0, R), jB = min(j1 - 1, dn - 1 - R);  // rows with an unclamped phi derivative
    bool lane_corner = false;
    if (edge) lane_corner = (c0 < dn) || (c0 + 3 >= dn + nx);
    const bool has_hl = (lane == 0) && (x0 > 0), has_hr = (lane == 31) && (x0 + TILE < pitch);

    auto issue = [&](int jl, int slot) {
        float4* st = ring + slot * SB_SIZE;
        const int y = yb0 + jl;
        const size_t ro = (size_t)y * pitch + xl;
        if (y + R <= nyt - 1) cp16(st + SB_P + lane, PC + (size_t)(y + R) * pitch + xl);
        cp16(st + SB_P1 + lane, P1 + ro);
        cp16(st + SB_C2 + lane, S.c2 + ro);
        cp16(st + SB_PY + lane, PHO + ro);
        cp16(st + SB_CY + lane, S.chy + ro);
        if (lane_corner) {
            cp16(st + SB_PX + lane, S.phx + ro);
            cp16(st + SB_CX + lane, S.chx + ro);
        }
        if (jl >= jA && jl <= jB) cp16(st + SB_FA + lane, PHO + (size_t)(yb0 + jl + R) * pitch + xl);
        if (has_hl) cp16(st + SB_HL, PC + (size_t)y * pitch + x0 - 4);
        if (has_hr) cp16(st + SB_HR, PC + (size_t)y * pitch + x0 + TILE);
    };
#pragma unroll
    for (int i = 0; i < BOT_DEPTH; ++i) {
        if (j0 + i < j1) issue(j0 + i, i);
        cp_commit();
    }

    // clamped values: rows jl < R use the phi derivative at local row R, rows
    // jl > dn-1-R that at dn-1-R (solver_space_derivs.f90:118-128 on the
    // strip); rows below nyt-1-R use the p derivatives of row nyt-1-R.
    float4 t[2 * R + 1];
    float dphyTop[4] = {0.f, 0.f, 0.f, 0.f}, dphyBot[4] = {0.f, 0.f, 0.f, 0.f};
    float d2yBot[4] = {0.f, 0.f, 0.f, 0.f}, dyBot[4] = {0.f, 0.f, 0.f, 0.f};
    if (j0 < R) {
#pragma unroll
        for (int i = 0; i <= 2 * R; ++i) t[i] = ld4(PHO + (size_t)(yb0 + i) * pitch + xl);
        yderiv1<R>(t, P, dphyTop);
    }
    if (j1 - 1 > dn - 1 - R) {
#pragma unroll
        for (int i = 0; i <= 2 * R; ++i) t[i] = ld4(PHO + (size_t)(nyt - 1 - 2 * R + i) * pitch + xl);
        yderiv1<R>(t, P, dphyBot);
#pragma unroll
        for (int i = 0; i <= 2 * R; ++i) t[i] = ldg4(PC + (size_t)(nyt - 1 - 2 * R + i) * pitch + xl);
        yderivs<R>(t, P, d2yBot, dyBot);
    }

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

    int ri = it.r0;
    int rrow = (ri < it.r1) ? P.recs[ri].row : INT_MAX;

    int slot = 0;
    for (int jl = j0; jl < j1; ++jl) {
        const int y = yb0 + jl;
        cp_wait<BOT_DEPTH - 1>();
        const float4* st = ring + slot * SB_SIZE;
        if (y + R <= nyt - 1) q[2 * R] = st[SB_P + lane];
        const size_t ro = (size_t)y * pitch + xl;
        float pm1[4], cc[4], pc[4];
        to_arr(st[SB_P1 + lane], pm1);
        to_arr(st[SB_C2 + lane], cc);
        to_arr(q[R], pc);
        float d2y[4], dy[4];
        if (y <= nyt - 1 - R) {
            yderivs<R>(q, P, d2y, dy);
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e) { d2y[e] = d2yBot[e]; dy[e] = dyBot[e]; }
        }
        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 hl = has_hl ? st[SB_HL] : z4, hr = has_hr ? st[SB_HR] : z4;
        float w[12];
        window(q[R], hl, hr, lane, w);
        float d2x[4], dx[4];
        xderivs<R>(w, P, d2x, dx);
        if (edge) xclamp<R>(S, x0, c0, first, last, d2x, dx);

        // strip-local y derivative of the old y-direction phi (pml_matrices_y :335)
        float dphy[4];
        if (jl < R) {
#pragma unroll
            for (int e = 0; e < 4; ++e) dphy[e] = dphyTop[e];
        } else if (jl <= dn - 1 - R) {
            f[2 * R] = st[SB_FA + lane];
            yderiv1<R>(f, P, dphy);
#pragma unroll
            for (int i = 0; i < 2 * R; ++i) f[i] = f[i + 1];
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e) dphy[e] = dphyBot[e];
        }

        float phy[4], chy[4];
        to_arr(st[SB_PY + lane], phy);
        to_arr(st[SB_CY + lane], chy);
        float phx[4] = {0.f, 0.f, 0.f, 0.f}, chx[4] = {0.f, 0.f, 0.f, 0.f}, dphx[4] = {0.f, 0.f, 0.f, 0.f};
        if (edge) {
            if (lane_corner) {
                to_arr(st[SB_PX + lane], phx);
                to_arr(st[SB_CX + lane], chx);
            }
            phi_xderiv<R>(S, P, from_arr(phx), lane, x0, c0, first, last, dphx);
        }

        float p3[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int c = c0 + e;
            if (c < 0 || c >= nxt) {
                p3[e] = 0.f;
                continue;
            }
            const bool left = c < dn, right = c >= dn + nx;
            // factor index: strip factor(j); corners factor(max(i,j)) with the
            // ld/rd orientation (solver_PML_coeffs.f90:240-267)
            int fi = jl;
            if (left) fi = max(jl, dn - 1 - c);
            if (right) fi = max(jl, c - dn - nx);
            const float A = __ldg(P.fA + fi), B = __ldg(P.fB + fi);
            const float phyn = A * phy[e] + B * dy[e];
            const float chyn = A * chy[e] + B * (d2y[e] + dphy[e]);
            const float propy = dphy[e] + chyn;
            phy[e] = phyn;
            chy[e] = chyn;
            if (!left && !right) {
                p3[e] = ((-pm1[e]) + 2.f * pc[e]) + cc[e] * ((d2x[e] + d2y[e]) + propy);
            } else {
                const float phxn = A * phx[e] + B * dx[e];
                const float chxn = A * chx[e] + B * (d2x[e] + dphx[e]);
                const float propx = dphx[e] + chxn;
                phx[e] = phxn;
                chx[e] = chxn;
                const float tt = ((-pm1[e]) + 2.f * pc[e]) + cc[e] * ((d2x[e] + d2y[e]) + propx);
                p3[e] = tt + cc[e] * propy;
            }
        }
        st4(PHN + ro, from_arr(phy));
        st4(S.chy + ro, from_arr(chy));
        if (lane_corner) {
            st4(S.phx + ro, from_arr(phx));
            st4(S.chx + ro, from_arr(chx));
        }
        st4(P1 + ro, from_arr(p3));
        if (MODE == 0 && P.record) record_row(P, S, y, xl, ri, it.r1, rrow, p3);

#pragma unroll
        for (int i = 0; i < 2 * R; ++i) q[i] = q[i + 1];
        if (jl + BOT_DEPTH < j1) issue(jl + BOT_DEPTH, slot);
        cp_commit();
        slot = (slot + 1 == BOT_DEPTH) ? 0 : slot + 1;
    }
    cp_wait<0>();
}

// Model rows of the middle tiles: interior cells only (no CPML, no clamp),
// so only second derivatives are needed.  This is the kernel that moves
// almost all of the bytes.  SNAP selects the variant for the time steps
// that store a snapshot (forward) or apply the imaging condition (adjoint);
// the adjoint variant also prefetches the snapshot row and the imaging
// accumulator row through the ring.
constexpr int IN_P = 0, IN_P1 = 32, IN_C2 = 64, IN_HL = 96, IN_HR = 97, IN_F = 98, IN_FS = 130, IN_K = 131;
constexpr int IN_SIZE = 98, IN_SIZE_IMG = 195;
constexpr int IN_DEPTH = 6, IN_DEPTH_IMG = 4;
constexpr int IN_SMEM = 4 * IN_DEPTH * IN_SIZE * 16;
constexpr int IN_SMEM_IMG = 4 * IN_DEPTH_IMG * IN_SIZE_IMG * 16;

__device__ __forceinline__ void cp4(void* smem_dst, const void* gmem_src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(gmem_src) : "memory");
}

template <int R, int MODE, bool SNAP>
__global__ void __launch_bounds__(128, (MODE == 1 && SNAP) ? 3 : 5) k_step_interior(const __grid_constant__ StepParams P) {
    constexpr bool IMG = (MODE == 1) && SNAP;
    constexpr int SZ = IMG ? IN_SIZE_IMG : IN_SIZE;
    constexpr int DEPTH = IMG ? IN_DEPTH_IMG : IN_DEPTH;
    extern __shared__ float4 smem[];
    const int lane = threadIdx.x & 31;
    const int wid = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (wid >= P.nitems) return;
    float4* ring = smem + (threadIdx.x >> 5) * (DEPTH * SZ);
    const WorkItem it = P.items[wid];
    const ShotDev& S = P.shots[it.shot];
    const int pitch = S.pitch;
    const int x0 = it.tile * TILE, xl = x0 + 4 * lane;
    const float* PC = (P.parity ? S.pa : S.pb) + xl;  // p at this lane's columns
    float* P1 = (P.parity ? S.pb : S.pa) + xl;        // p_1, overwritten with p_3
    const float* C2 = S.c2 + xl;
    // every middle tile has both neighbours; lanes 0 and 31 fetch the halos
    const int hoff = (lane == 0) ? -4 - 4 * lane : TILE - 4 * lane;
    const bool has_h = (lane == 0) || (lane == 31);
    float4* hslot = ring + (lane == 0 ? IN_HL : IN_HR);
    const size_t snap_base = IMG ? (size_t)P.snap * (size_t)S.snap_stride : 0;

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
                    cp4(st + IN_FS, S.sscale + ((size_t)P.snap * S.ny + (y - S.dn)) * S.ntiles + it.tile);
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
        float w[12];
        window(q[R], h, h, lane, w);
        float d2x[4], d2y[4];
        xderiv2<R>(w, P, d2x);
        yderiv2<R>(q, P, d2y);

        // source injection: source(nys,nxs) = S(k-1,j)  (solver_acoustic_SS.f90:319-330)
        float sv[4] = {0.f, 0.f, 0.f, 0.f};
        while (srow == y) {
            const SrcEnt s = P.srcs[si];
            if ((s.col >> 2) == (xl >> 2)) {
                const float val = __ldg(S.srcv + (size_t)s.vidx * S.nt + P.t);
                const int el = s.col & 3;
                sv[0] = el == 0 ? val : sv[0];
                sv[1] = el == 1 ? val : sv[1];
                sv[2] = el == 2 ? val : sv[2];
                sv[3] = el == 3 ? val : sv[3];
            }
            ++si;
            srow = (si < it.s1) ? P.srcs[si].row : INT_MAX;
        }
        // p_3 = -p_1 + 2p + (d2x + d2y + source)*c2  (:433-434)
        float p3[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) p3[e] = ((-pm1[e]) + 2.f * pc[e]) + (((d2x[e] + d2y[e]) + sv[e]) * cc[e]);

        if (MODE == 0 && SNAP) store_snapshot(P, S, y - S.dn, lane, x0, xl, xl - S.off, p3, pm1, it.tile);
        if (IMG) {
            // kernel += -0.5*(p_3-p_1)*Fields(snap)*store_snap  (:465-466); all columns interior
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
                st4(S.k32 + ko, k);
            } else {
                const double2* kk = reinterpret_cast<const double2*>(st + IN_K) + 2 * lane;
                double2 a = kk[0], b = kk[1];
                a.x += (double)k2[0]; a.y += (double)k2[1]; b.x += (double)k2[2]; b.y += (double)k2[3];
                double2* K2 = reinterpret_cast<double2*>(S.k64 + ko);
                K2[0] = a;
                K2[1] = b;
            }
        }
        st4(P1 + (size_t)y * pitch, from_arr(p3));
        if (MODE == 0 && P.record) record_row(P, S, y, xl, ri, it.r1, rrow, p3);

#pragma unroll
        for (int i = 0; i < 2 * R; ++i) q[i] = q[i + 1];
        if (y + DEPTH < it.y1) issue(y + DEPTH, slot);
        cp_commit();
        slot = (slot + 1 == DEPTH) ? 0 : slot + 1;
    }
    cp_wait<0>();
}

// Everything next to a boundary: model rows of the first/last tile (kind 0)
// and the bottom pad rows of every tile (kind 1).  Runs on a second stream,
// concurrently with k_step_interior.
constexpr int BND_WARP_F4 = (MAIN_DEPTH * ST_SIZE > BOT_DEPTH * SB_SIZE) ? MAIN_DEPTH * ST_SIZE : BOT_DEPTH * SB_SIZE;
constexpr int BND_SMEM = 4 * BND_WARP_F4 * 16;

template <int R, int MODE>
__global__ void __launch_bounds__(128) k_step_boundary(const __grid_constant__ StepParams P) {
    extern __shared__ float4 smem[];
    const int lane = threadIdx.x & 31;
    const int wid = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (wid >= P.nitems) return;
    float4* ring = smem + (threadIdx.x >> 5) * BND_WARP_F4;
    const WorkItem it = P.items[wid];
    if (it.kind == 0) edge_rows<R, MODE>(P, it, ring, lane);
    else bottom_rows<R, MODE>(P, it, ring, lane);
}

// Opt the step kernels into the dynamic shared memory they use (the
// boundary kernel's prefetch rings are above the 48 KB default).
cudaError_t configure_step_kernels() {
    cudaError_t e = cudaSuccess;
#define FWI_CFG(R_, M_)                                                                                           \
    if (e == cudaSuccess)                                                                                         \
        e = cudaFuncSetAttribute(k_step_interior<R_, M_, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,      \
                                 IN_SMEM);                                                                         \
    if (e == cudaSuccess)                                                                                         \
        e = cudaFuncSetAttribute(k_step_interior<R_, M_, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,       \
                                 M_ == 1 ? IN_SMEM_IMG : IN_SMEM);                                                 \
    if (e == cudaSuccess)                                                                                         \
        e = cudaFuncSetAttribute(k_step_boundary<R_, M_>, cudaFuncAttributeMaxDynamicSharedMemorySize, BND_SMEM);
    FWI_CFG(3, 0)
    FWI_CFG(3, 1)
    FWI_CFG(4, 0)
    FWI_CFG(4, 1)
#undef FWI_CFG
    return e;
}

// Interior kernel on stream sm and boundary kernel on stream sb (the caller
// orders the two streams around each time step).
cudaError_t launch_step(int acc, int mode, const StepParams& pm, const StepParams& pb, cudaStream_t sm,
                        cudaStream_t sb) {
    const int bm = (pm.nitems + 3) / 4, bb = (pb.nitems + 3) / 4;
#define FWI_LAUNCH(R_, M_)                                                          \
    do {                                                                           \
        if (bb) k_step_boundary<R_, M_><<<bb, 128, BND_SMEM, sb>>>(pb);             \
        if (bm) {                                                                  \
            if (pm.snap >= 0)                                                      \
                k_step_interior<R_, M_, true><<<bm, 128, M_ == 1 ? IN_SMEM_IMG : IN_SMEM, sm>>>(pm); \
            else                                                                   \
                k_step_interior<R_, M_, false><<<bm, 128, IN_SMEM, sm>>>(pm);      \
        }                                                                          \
    } while (0)
    if (acc == 3) {
        if (mode == 0) FWI_LAUNCH(3, 0);
        else FWI_LAUNCH(3, 1);
    } else if (acc == 4) {
        if (mode == 0) FWI_LAUNCH(4, 0);
        else FWI_LAUNCH(4, 1);
    } else {
        return cudaErrorInvalidValue;
    }
#undef FWI_LAUNCH
    return cudaGetLastError();
}

}  // namespace fwi
