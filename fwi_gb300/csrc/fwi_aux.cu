// Auxiliary kernels of the FWI path: model padding (c2), misfit and adjoint
// source, gradient stacking/finalisation, layout conversion for the
// drop-in solver entry point, and the FP64 dot products of Beta_calculous.
// Compiled with --fmad=false (see fwi_step.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "fwi_internal.cuh"

namespace fwi {

namespace {

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Padded c2 = c**2*dt**2/d**2 (solver_acoustic_SS.f90:271-292).  The padded
// velocity copies the nearest model cell, i.e. clamps the model indices.
// Source velocity: vp(ny, ldv) column-major starting at column x0, or, when
// from_lambda, vp = sqrt(lambda/1000.) (calculate_misfit_gradient.f90:252).
__global__ void k_build_c2(float* c2, int nyt, int pitch, int off, int dn, int ny, int nx, const float* src, int ldv,
                           int x0, int from_lambda, float dt2, float d2) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;  // physical column
    const int y = blockIdx.y;
    if (x >= pitch || y >= nyt) return;
    const int c = x - off;
    float out = 0.f;
    const int nxt = nx + 2 * dn;
    if (c >= 0 && c < nxt) {
        const int my = min(max(y - dn, 0), ny - 1), mx = min(max(c - dn, 0), nx - 1);
        float v = src[(size_t)my + (size_t)(x0 + mx) * ldv];
        if (from_lambda) v = __fsqrt_rn(__fdiv_rn(v, 1000.f));
        out = __fdiv_rn(__fmul_rn(__fmul_rn(v, v), dt2), d2);
    }
    c2[(size_t)y * pitch + x] = out;
}

// Rec_point(nt,:) = Rec_point(nt-1,:)  (solver_acoustic_SS.f90:588)
__global__ void k_rec_last(float* rec, int nt, int nrec) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nrec && nt >= 2) rec[(size_t)i * nt + nt - 1] = rec[(size_t)i * nt + nt - 2];
}

// Misfit_function + Misfit_L2 for one trace per block (Misfit.f90:31-61,
// Misfit_L2.f90:8-14).  r(k) = S(k)/maxS - T(k)/maxT in FP32 when the
// observed trace is nonzero and both maxima are nonzero, else 0;
// misfit_tr = sum 0.5*dt*r^2 in FP64; adj(k) = -r(nt-k+1).
__global__ void k_misfit_trace(const float* synth, const float* obs, float* adj, double* mis_tr, int nt, float dt,
                               const int* tr_off, int ntr_total) {
    const int tr = blockIdx.x;
    if (tr >= ntr_total) return;
    const float* s = synth + (size_t)tr * nt;
    const float* o = obs + (size_t)tr * nt;
    float* a = adj + (size_t)tr * nt;
    __shared__ float sh_ms[32], sh_mt[32];
    __shared__ int sh_nz[32];
    __shared__ double sh_sum[32];
    float ms = 0.f, mt = 0.f;
    int nz = 0;
    for (int k = threadIdx.x; k < nt; k += blockDim.x) {
        const float sv = s[k], ov = o[k];
        ms = fmaxf(ms, fabsf(sv));
        mt = fmaxf(mt, fabsf(ov));
        nz |= (ov != 0.f);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    ms = warp_max(ms);
    mt = warp_max(mt);
    nz = __any_sync(0xffffffffu, nz);
    if (lane == 0) { sh_ms[w] = ms; sh_mt[w] = mt; sh_nz[w] = nz; }
    __syncthreads();
    if (threadIdx.x == 0) {
        float a1 = 0.f, a2 = 0.f;
        int z = 0;
        for (int i = 0; i < nw; ++i) { a1 = fmaxf(a1, sh_ms[i]); a2 = fmaxf(a2, sh_mt[i]); z |= sh_nz[i]; }
        sh_ms[0] = a1; sh_mt[0] = a2; sh_nz[0] = z;
    }
    __syncthreads();
    const float maxS = sh_ms[0], maxT = sh_mt[0];
    const bool use = sh_nz[0] && maxS != 0.f && maxT != 0.f;
    double acc = 0.0;
    const double hdt = 0.5 * (double)dt;
    for (int k = threadIdx.x; k < nt; k += blockDim.x) {
        // residual of the sample mirrored in time goes to adj(k)
        const int km = nt - 1 - k;
        float r = 0.f, rm = 0.f;
        if (use) {
            r = __fsub_rn(__fdiv_rn(s[k], maxS), __fdiv_rn(o[k], maxT));
            rm = __fsub_rn(__fdiv_rn(s[km], maxS), __fdiv_rn(o[km], maxT));
        }
        acc += hdt * (double)r * (double)r;
        a[k] = -rm;
    }
    acc = warp_sum(acc);
    __syncthreads();
    if (lane == 0) sh_sum[w] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < nw; ++i) t += sh_sum[i];
        mis_tr[tr] = t;
    }
    (void)tr_off;
}

// Per-shot misfit: sum of the shot's traces in receiver order.
__global__ void k_misfit_shots(const double* mis_tr, const int* tr_off, int nshots, double* mis_shot) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nshots) return;
    double t = 0.0;
    for (int i = tr_off[s]; i < tr_off[s + 1]; ++i) t += mis_tr[i];
    mis_shot[s] = t;
}

// Stack the wave's per-shot imaging accumulators into the model-size FP64
// gradient G(ny, nxm) (column-major), shots in index order.
struct StackShot {
    const float* k32;
    const double* k64;
    int x0, nx, off_dn, pitch;
    double w;
};
__global__ void k_stack(double* G, int ny, int nxm, const StackShot* shots, int nshots, int form) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;  // model column
    const int j = blockIdx.y * blockDim.y + threadIdx.y;  // row
    if (i >= nxm || j >= ny) return;
    double g = G[(size_t)j + (size_t)i * ny];
    for (int s = 0; s < nshots; ++s) {
        const StackShot& sh = shots[s];
        const int li = i - sh.x0;
        if (li < 0 || li >= sh.nx) continue;
        const size_t o = (size_t)j * sh.pitch + sh.off_dn + li;
        const double v = form ? sh.k64[o] : (double)sh.k32[o];
        g += sh.w * v;
    }
    G[(size_t)j + (size_t)i * ny] = g;
}

// Grad = Grad + G/numtasks, then Grad(1:k(i), i) = 0
// (calculate_misfit_gradient.f90:342-351).
__global__ void k_finalize(float* grad, const double* G, int ny, int nxm, int numtasks, const int* water) {
    const size_t n = (size_t)ny * nxm;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(idx % ny), i = (int)(idx / ny);
        float v = __fadd_rn(grad[idx], (float)(G[idx] / (double)numtasks));
        if (water && j < water[i]) v = 0.f;
        grad[idx] = v;
    }
}

// Fields(ny, nx*(nsnap)) Fortran <-> device snapshot store [s][ny][pitch].
__global__ void k_fields_to_fortran(float* out, const float* snaps, int ny, int nx, int pitch, int off_dn, int nsnap) {
    const size_t n = (size_t)ny * nx * nsnap;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(idx % ny);
        const size_t col = idx / ny;  // s*nx + i
        const int s = (int)(col / nx), i = (int)(col % nx);
        out[idx] = snaps[((size_t)s * ny + j) * pitch + off_dn + i];
    }
}
__global__ void k_fields_from_fortran(float* snaps, const float* in, int ny, int nx, int pitch, int off_dn, int nsnap) {
    const size_t n = (size_t)ny * nx * nsnap;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(idx % ny);
        const size_t col = idx / ny;
        const int s = (int)(col / nx), i = (int)(col % nx);
        snaps[((size_t)s * ny + j) * pitch + off_dn + i] = in[idx];
    }
}
// kernel(ny,nx) Fortran <-> device accumulator [ny][pitch]
__global__ void k_kernel_io(float* dev, float* fort, int ny, int nx, int pitch, int off_dn, int to_dev) {
    const size_t n = (size_t)ny * nx;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(idx % ny), i = (int)(idx / ny);
        float* d = dev + (size_t)j * pitch + off_dn + i;
        if (to_dev) *d = fort[idx];
        else fort[idx] = *d;
    }
}

// Beta_calculous (Beta_calculous.f90:10-22): Num = sum g*(g-o), Den = sum o*o
// in FP64; one partial per block, summed in block order by k_dot_final.
__global__ void k_dot_partial(const float* g, const float* o, size_t n, double* part) {
    double a = 0.0, b = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double gv = g[i], ov = o[i];
        a += gv * (gv - ov);
        b += ov * ov;
    }
    __shared__ double sa[32], sb[32];
    a = warp_sum(a);
    b = warp_sum(b);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { sa[w] = a; sb[w] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0, y = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) { x += sa[i]; y += sb[i]; }
        part[2 * blockIdx.x] = x;
        part[2 * blockIdx.x + 1] = y;
    }
}
__global__ void k_dot_final(const double* part, int nb, double* out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double x = 0.0, y = 0.0;
        for (int i = 0; i < nb; ++i) { x += part[2 * i]; y += part[2 * i + 1]; }
        out[0] = x;
        out[1] = y;
    }
}

// Copy many equal-purpose buffers in one launch (checkpoint save/restore of
// the wavefield state): job j copies n4 float4 from src to dst.
struct CopyJob {
    const float4* src;
    float4* dst;
    size_t n4;
};
__global__ void k_copy_jobs(const CopyJob* jobs, int njobs) {
    for (int j = blockIdx.y; j < njobs; j += gridDim.y) {
        const CopyJob c = jobs[j];
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < c.n4; i += (size_t)gridDim.x * blockDim.x)
            c.dst[i] = c.src[i];
    }
}

// Non-finite detector over a float array (sets *flag = 1).
__global__ void k_nonfinite(const float* a, size_t n, int* flag) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        if (!isfinite(a[i])) { *flag = 1; return; }
}

// The NLCG model arithmetic of FWI.f90 in the reference's FP32 operations,
// with exp and log evaluated in FP64 and rounded once to FP32 (the correctly
// rounded value of the FP32 function).
//
// max|Search/log(var_orig)| (FWI.f90:175): per element the FP32 log, the
// FP32 quotient and its magnitude; the maximum over all elements (NaN
// entries skipped, as MAXVAL compares with >) as the bits of a non-negative
// float, which order like integers.
__global__ void k_search_max(const float* search, const float* var, size_t n, unsigned* out) {
    float m = 0.f;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float lg = __double2float_rn(log((double)var[i]));
        const float v = fabsf(__fdiv_rn(search[i], lg));
        if (v > m) m = v;
    }
    m = warp_max(m);
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

// lambda = exp(Search*step)*var_orig (FWI.f90:227, :315): FP32 product, exp,
// FP32 product.
__global__ void k_model_update(const float* search, const float* var, float step, size_t n, float* lam) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float t = __fmul_rn(search[i], step);
        const float e = __double2float_rn(exp((double)t));
        lam[i] = __fmul_rn(e, var[i]);
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers used by the host code
// ---------------------------------------------------------------------------

cudaError_t launch_build_c2(float* c2, int nyt, int pitch, int off, int dn, int ny, int nx, const float* src, int ldv,
                            int x0, int from_lambda, float dt2, float d2, cudaStream_t st) {
    dim3 b(128, 1), g((pitch + 127) / 128, nyt);
    k_build_c2<<<g, b, 0, st>>>(c2, nyt, pitch, off, dn, ny, nx, src, ldv, x0, from_lambda, dt2, d2);
    return cudaGetLastError();
}
cudaError_t launch_rec_last(float* rec, int nt, int nrec, cudaStream_t st) {
    if (nrec <= 0) return cudaSuccess;
    k_rec_last<<<(nrec + 127) / 128, 128, 0, st>>>(rec, nt, nrec);
    return cudaGetLastError();
}
cudaError_t launch_misfit(const float* synth, const float* obs, float* adj, double* mis_tr, int nt, float dt,
                          const int* tr_off, int ntr, int nshots, double* mis_shot, cudaStream_t st) {
    if (ntr > 0) k_misfit_trace<<<ntr, 256, 0, st>>>(synth, obs, adj, mis_tr, nt, dt, tr_off, ntr);
    if (nshots > 0) k_misfit_shots<<<(nshots + 127) / 128, 128, 0, st>>>(mis_tr, tr_off, nshots, mis_shot);
    return cudaGetLastError();
}
cudaError_t launch_stack(double* G, int ny, int nxm, const void* shots, int nshots, int form, cudaStream_t st) {
    dim3 b(32, 8), g((nxm + 31) / 32, (ny + 7) / 8);
    k_stack<<<g, b, 0, st>>>(G, ny, nxm, reinterpret_cast<const StackShot*>(shots), nshots, form);
    return cudaGetLastError();
}
size_t stack_shot_size() { return sizeof(StackShot); }
void fill_stack_shot(void* dst, const float* k32, const double* k64, int x0, int nx, int off_dn, int pitch, double w) {
    StackShot s{k32, k64, x0, nx, off_dn, pitch, w};
    *reinterpret_cast<StackShot*>(dst) = s;
}
cudaError_t launch_finalize(float* grad, const double* G, int ny, int nxm, int numtasks, const int* water,
                            cudaStream_t st) {
    k_finalize<<<1024, 256, 0, st>>>(grad, G, ny, nxm, numtasks, water);
    return cudaGetLastError();
}
cudaError_t launch_fields_io(float* fort, float* snaps, int ny, int nx, int pitch, int off_dn, int nsnap, int to_dev,
                             cudaStream_t st) {
    if (to_dev) k_fields_from_fortran<<<2048, 256, 0, st>>>(snaps, fort, ny, nx, pitch, off_dn, nsnap);
    else k_fields_to_fortran<<<2048, 256, 0, st>>>(fort, snaps, ny, nx, pitch, off_dn, nsnap);
    return cudaGetLastError();
}
cudaError_t launch_kernel_io(float* dev, float* fort, int ny, int nx, int pitch, int off_dn, int to_dev,
                             cudaStream_t st) {
    k_kernel_io<<<512, 256, 0, st>>>(dev, fort, ny, nx, pitch, off_dn, to_dev);
    return cudaGetLastError();
}
cudaError_t launch_dot(const float* g, const float* o, size_t n, double* part, int nb, double* out, cudaStream_t st) {
    k_dot_partial<<<nb, 256, 0, st>>>(g, o, n, part);
    k_dot_final<<<1, 32, 0, st>>>(part, nb, out);
    return cudaGetLastError();
}
cudaError_t launch_search_max(const float* search, const float* var, size_t n, unsigned* out, cudaStream_t st) {
    k_search_max<<<2 * 152, 256, 0, st>>>(search, var, n, out);
    return cudaGetLastError();
}
cudaError_t launch_model_update(const float* search, const float* var, float step, size_t n, float* lam,
                                cudaStream_t st) {
    k_model_update<<<4 * 152, 256, 0, st>>>(search, var, step, n, lam);
    return cudaGetLastError();
}
size_t copy_job_size() { return sizeof(CopyJob); }
void fill_copy_job(void* dst, const void* src, void* to, size_t bytes) {
    CopyJob c{reinterpret_cast<const float4*>(src), reinterpret_cast<float4*>(to), bytes / 16};
    *reinterpret_cast<CopyJob*>(dst) = c;
}
cudaError_t launch_copy_jobs(const void* jobs, int njobs, cudaStream_t st) {
    if (njobs <= 0) return cudaSuccess;
    dim3 g(64, (unsigned)std::min(njobs, 65535));
    k_copy_jobs<<<g, 256, 0, st>>>(reinterpret_cast<const CopyJob*>(jobs), njobs);
    return cudaGetLastError();
}
cudaError_t launch_nonfinite(const float* a, size_t n, int* flag, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_nonfinite<<<256, 256, 0, st>>>(a, n, flag);
    return cudaGetLastError();
}

}  // namespace fwi
