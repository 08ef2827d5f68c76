// Per-shot pre-processing of traces on the device: the frequency filter and
// the resampling to the modelling time step that calculate_misfit_gradient
// applies to the observed data and the source before every solver call
// (calculate_misfit_gradient.f90:193-194, :241-244).
//
//   fwi_time_filter          time_filter (time_filter.f90:1-40) with the
//                            Butterworth response of filters_function1D
//                            (filters.f90:39-186): each trace is placed at
//                            the end of a 24x zero-padded buffer, transformed,
//                            multiplied by H(f) and transformed back.
//   fwi_interpolation_akima  interpolation_akima (interpolation_akima.f90:1-31)
//                            with Akima's local cubic (ACM Algorithm 433,
//                            Comm. ACM 15(10):914, 1972; akima433.f90:6-170),
//                            one thread per output sample.
//
// This file is compiled with --fmad=false: the Akima arithmetic is evaluated
// in the order of the Fortran source, in FP32, so the resampled traces are
// bit-identical to the reference's.  The filter's FFT is cuFFT in FP32 (the
// reference uses FFTPACK5 in FP32); its results agree to rounding.
#include <cuda_runtime.h>
#include <cufft.h>

#include <cmath>
#include <complex>
#include <vector>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "fwi_gb300.h"

namespace fwi {

int prep_fail(int code, const std::string& msg);      // fwi_host.cu
cudaStream_t prep_stream();                           // fwi_host.cu
bool prep_is_device_ptr(const void* p);               // fwi_host.cu
int prep_ensure_init();                               // fwi_host.cu

namespace {

// --------------------------------------------------------------------------
// Akima interpolation (one thread per output sample)
// --------------------------------------------------------------------------

// Abscissa i (1-based) of a uniform axis: real(i-1)*dt, as the reference
// builds Time_Data and time (interpolation_akima.f90:14-20).
__host__ __device__ __forceinline__ float axis(int i, float d) { return (float)(i - 1) * d; }

// Abscissae for the interpolation below: a uniform axis, or the values of an
// array x(1..L).  The evaluation is compiled for the device (trace
// resampling) and for the host (the WAS bathymetry model of the geometry).
struct UniformAxis {
    float d;
    __host__ __device__ float operator()(int i) const { return axis(i, d); }
};
struct ArrayAxis {
    const float* x;
    __host__ __device__ float operator()(int i) const { return x[i - 1]; }
};

// Interval index I of u among x(1..L) (x strictly increasing): 1 before
// x(1), L+1 at or after x(L), else the smallest i >= 2 with x(i) > u, found
// by the same bisection (akima433.f90, the routine that locates the point).
template <typename AX>
__host__ __device__ __forceinline__ int akima_interval(float u, int L, AX ax) {
    if (L == 2) return 2;
    if (u >= ax(L)) return L + 1;
    if (u < ax(1)) return 1;
    int lo = 2, hi = L;
    do {
        const int i = (lo + hi) / 2;
        if (u >= ax(i)) lo = i + 1;
        else hi = i;
    } while (hi > lo);
    return hi;
}

// Value at u of Akima's piecewise cubic through (x(i), y(i)), i = 1..L.
// Slopes of the five intervals around the one holding u (missing ones at the
// ends extrapolated linearly), Akima's weighted slope estimates at the two
// interval ends, and the cubic through them; before x(1) and after x(L) the
// end interval's cubic is shifted outward as in the reference.
template <typename AX>
__host__ __device__ float akima_eval(const float* y, int L, AX ax, float u) {
    const int I = akima_interval(u, L, ax);
    int J = I;
    if (J == 1) J = 2;
    if (J == L + 1) J = L;
    float x3 = ax(J - 1), y3 = y[J - 2];
    const float x4 = ax(J), y4 = y[J - 1];
    float a3 = x4 - x3;
    float m3 = (y4 - y3) / a3;
    float a2 = 0.f, a4 = 0.f, m1, m2 = 0.f, m4, m5;
    float x2 = 0.f, y2 = 0.f, x5 = 0.f, y5 = 0.f;
    if (L == 2) {
        m2 = m3;
        m4 = m3;
    } else {
        if (J != 2) {
            x2 = ax(J - 2);
            y2 = y[J - 3];
            a2 = x3 - x2;
            m2 = (y3 - y2) / a2;
        }
        if (J == L) {
            m4 = m3 + m3 - m2;
        } else {
            x5 = ax(J + 1);
            y5 = y[J];
            a4 = x5 - x4;
            m4 = (y5 - y4) / a4;
            if (J == 2) m2 = m3 + m3 - m4;
        }
    }
    if (J <= 3) {
        m1 = m2 + m2 - m3;
    } else {
        const float a1 = x2 - ax(J - 3);
        m1 = (y2 - y[J - 4]) / a1;
    }
    if (J >= L - 1) {
        m5 = m4 + m4 - m3;
    } else {
        const float a5 = ax(J + 2) - x5;
        m5 = (y[J + 1] - y5) / a5;
    }
    // numerical differentiation: slope estimates t3 (left end), t4 (right end)
    float t3 = 0.f, t4;
    if (I != L + 1) {
        float w2 = fabsf(m4 - m3), w3 = fabsf(m2 - m1), sw = w2 + w3;
        if (sw == 0.f) {
            w2 = 0.5f;
            w3 = 0.5f;
            sw = 1.f;
        }
        t3 = (w2 * m2 + w3 * m3) / sw;
    }
    if (I == 1) {
        t4 = t3;
        const float sa = a3 + a4;
        t3 = 0.5f * (m1 + m2 - a4 * (a3 - a4) * (m3 - m4) / (sa * sa));
        x3 = x3 - a4;
        y3 = y3 - m2 * a4;
        a3 = a4;
        m3 = m2;
    } else {
        float w3 = fabsf(m5 - m4), w4 = fabsf(m3 - m2), sw = w3 + w4;
        if (sw == 0.f) {
            w3 = 0.5f;
            w4 = 0.5f;
            sw = 1.f;
        }
        t4 = (w3 * m3 + w4 * m4) / sw;
        if (I == L + 1) {
            t3 = t4;
            const float sa = a2 + a3;
            t4 = 0.5f * (m4 + m5 - a2 * (a2 - a3) * (m2 - m3) / (sa * sa));
            x3 = x4;
            y3 = y4;
            a3 = a2;
            m3 = m4;
        }
    }
    // coefficients of the cubic and its value
    const float q2 = (2.0f * (m3 - t3) + m3 - t4) / a3;
    const float q3 = (-m3 - m3 + t3 + t4) / (a3 * a3);
    const float d = u - x3;
    return y3 + d * (t3 + d * (q2 + d * q3));
}

__global__ void k_akima(const float* __restrict__ in, int nt_in, float dt_in, float* __restrict__ out, int nt_out,
                        float dt_out, int ntr) {
    const long long n = (long long)nt_out * ntr;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int tr = (int)(idx / nt_out), k = (int)(idx % nt_out);
        out[idx] = akima_eval(in + (size_t)tr * nt_in, nt_in, UniformAxis{dt_in}, axis(k + 1, dt_out));
    }
}

// --------------------------------------------------------------------------
// Butterworth filter in the frequency domain
// --------------------------------------------------------------------------

// Butterworth response H at the frequencies j*fe/ts, j = 0..ts/2, for the
// filter types of filters_function1D (1 low-pass at fc, 2 high-pass at fs =
// 40 Hz, 3 band-pass between f1 and fc) and order n.  As in the reference the
// even-order product over k = 1..n/2 is used for every n (parity = 0 there),
// the frequency advances by an FP32 accumulation of fe/ts, and H(0) is 1 for
// the low-pass and 0 otherwise (filters.f90:88-181).  The products are formed
// in double precision.
std::vector<std::complex<double>> butterworth_response(int n, int typef, float fc, float f1, float fe, int ts) {
    const float fs = 40.f, f2 = fc;
    const float f0 = std::sqrt(f1 * f2), Q = f0 / (f2 - f1);
    const double pi = 3.14159265;  // the reference's constant
    const std::complex<double> I(0.0, 1.0);
    std::vector<std::complex<double>> H(ts / 2 + 1);
    float f = 0.f;
    const float df = fe / (float)ts;
    for (int j = 0; j <= ts / 2; ++j) {
        std::complex<double> B(1.0, 0.0);
        for (int k = 1; k <= n / 2; ++k) {
            const double c = std::cos((double)(2 * k + n - 1) * pi / (2.0 * n));
            std::complex<double> s;
            if (typef == 1) s = I * (double)f / (double)fc;
            else if (typef == 2) s = (double)fs / (I * (double)f);
            else s = (double)Q * ((I * (double)f) / (double)f0 + (double)f0 / (I * (double)f));
            B *= s * s - 2.0 * s * c + 1.0;
        }
        H[j] = 1.0 / B;
        f = f + df;
    }
    H[0] = (typef == 1) ? 1.0 : 0.0;
    return H;
}

__global__ void k_pad_traces(const float* __restrict__ in, int nt, int ntr, float* __restrict__ buf, int ts) {
    const long long n = (long long)ts * ntr;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int tr = (int)(idx / ts), j = (int)(idx % ts);
        buf[idx] = (j >= ts - nt) ? in[(size_t)tr * nt + (j - (ts - nt))] : 0.f;
    }
}

__global__ void k_apply_response(cufftComplex* __restrict__ Z, const float2* __restrict__ H, int nf, int ntr) {
    const long long n = (long long)nf * ntr;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        const float2 h = H[idx % nf];
        const cufftComplex z = Z[idx];
        Z[idx] = make_float2(z.x * h.x - z.y * h.y, z.x * h.y + z.y * h.x);
    }
}

__global__ void k_unpad_traces(const float* __restrict__ buf, int ts, int nt, int ntr, float* __restrict__ out) {
    const long long n = (long long)nt * ntr;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int tr = (int)(idx / nt), k = (int)(idx % nt);
        out[idx] = buf[(size_t)tr * ts + (ts - nt) + k];
    }
}

int grid_for(long long n) { return (int)std::max(1LL, std::min((n + 255) / 256, 152LL * 32)); }

struct Scratch {
    void* p = nullptr;
    size_t n = 0;
    ~Scratch() {
        if (p) cudaFree(p);
    }
    int ensure(size_t bytes) {
        if (p && n >= bytes) return FWI_OK;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        if (cudaMalloc(&p, bytes) != cudaSuccess) {
            cudaGetLastError();
            return prep_fail(FWI_ERR_NOMEM, "cudaMalloc failed for the filter scratch");
        }
        n = bytes;
        return FWI_OK;
    }
};

struct PrepState {
    std::mutex mu;
    int order = 6;  // filters.f90:21
    Scratch traces, out, buf, spec, resp;
    std::map<std::pair<int, int>, std::pair<cufftHandle, cufftHandle>> plans;  // (ts, batch) -> (R2C, C2R)
    ~PrepState() {
        for (auto& kv : plans) {
            cufftDestroy(kv.second.first);
            cufftDestroy(kv.second.second);
        }
    }
};
PrepState& PS() {
    static PrepState s;
    return s;
}

#define PCK(x)                                                                                          \
    do {                                                                                                \
        cudaError_t e_ = (x);                                                                           \
        if (e_ != cudaSuccess) return prep_fail(FWI_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)
#define PFT(x)                                                                                          \
    do {                                                                                                \
        cufftResult r_ = (x);                                                                           \
        if (r_ != CUFFT_SUCCESS) return prep_fail(FWI_ERR_CUDA, std::string(#x) + " failed (cuFFT " + std::to_string((int)r_) + ")"); \
    } while (0)
#define PTRY(x)                    \
    do {                           \
        int r_ = (x);              \
        if (r_ != FWI_OK) return r_; \
    } while (0)

}  // namespace

// Filter `ntr` device traces (nt, ntr) in place.
int filter_traces_device(float* d, int nt, float dt, int ntr, int typef, float f1, float fc) {
    PrepState& S = PS();
    const int zero_pad = 24;  // time_filter.f90:12
    const long long ts = (long long)zero_pad * nt;
    if (ts > (1LL << 30)) return prep_fail(FWI_ERR_ARG, "trace too long for the filter");
    const int nf = (int)(ts / 2 + 1);
    const float fe = 1.f / dt;
    std::vector<std::complex<double>> H = butterworth_response(S.order, typef, fc, f1, fe, (int)ts);
    // forward transform normalised by 1/ts as FFTPACK5's; the inverse is not.
    // The output keeps the real part: only the Hermitian part of the product
    // contributes, so the Nyquist bin takes Re(H).
    std::vector<float2> h(nf);
    for (int j = 0; j < nf; ++j) {
        std::complex<double> v = H[j] / (double)ts;
        if (j == nf - 1) v = std::complex<double>(v.real(), 0.0);
        h[j] = make_float2((float)v.real(), (float)v.imag());
    }
    cudaStream_t st = prep_stream();
    PTRY(S.resp.ensure((size_t)nf * sizeof(float2)));
    PCK(cudaMemcpyAsync(S.resp.p, h.data(), (size_t)nf * sizeof(float2), cudaMemcpyHostToDevice, st));
    // batches of traces within about 1 GB of scratch
    const size_t per_trace = (size_t)ts * 4 + (size_t)nf * 8;
    const int batch = (int)std::max<size_t>(1, std::min<size_t>((size_t)ntr, (1ull << 30) / per_trace));
    PTRY(S.buf.ensure((size_t)batch * ts * 4));
    PTRY(S.spec.ensure((size_t)batch * nf * 8));
    for (int t0 = 0; t0 < ntr; t0 += batch) {
        const int nb = std::min(batch, ntr - t0);
        auto key = std::make_pair((int)ts, nb);
        auto it = S.plans.find(key);
        if (it == S.plans.end()) {
            cufftHandle fwd, inv;
            int len = (int)ts;
            PFT(cufftPlanMany(&fwd, 1, &len, nullptr, 1, len, nullptr, 1, nf, CUFFT_R2C, nb));
            PFT(cufftPlanMany(&inv, 1, &len, nullptr, 1, nf, nullptr, 1, len, CUFFT_C2R, nb));
            it = S.plans.emplace(key, std::make_pair(fwd, inv)).first;
        }
        PFT(cufftSetStream(it->second.first, st));
        PFT(cufftSetStream(it->second.second, st));
        float* buf = reinterpret_cast<float*>(S.buf.p);
        cufftComplex* Z = reinterpret_cast<cufftComplex*>(S.spec.p);
        float* tr = d + (size_t)t0 * nt;
        k_pad_traces<<<grid_for(ts * nb), 256, 0, st>>>(tr, nt, nb, buf, (int)ts);
        PCK(cudaGetLastError());
        PFT(cufftExecR2C(it->second.first, buf, Z));
        k_apply_response<<<grid_for((long long)nf * nb), 256, 0, st>>>(Z, reinterpret_cast<const float2*>(S.resp.p),
                                                                       nf, nb);
        PCK(cudaGetLastError());
        PFT(cufftExecC2R(it->second.second, Z, buf));
        k_unpad_traces<<<grid_for((long long)nt * nb), 256, 0, st>>>(buf, (int)ts, nt, nb, tr);
        PCK(cudaGetLastError());
    }
    return FWI_OK;
}

int akima_device(const float* din, int nt_in, float dt_in, float* dout, int nt_out, float dt_out, int ntr) {
    cudaStream_t st = prep_stream();
    const long long n = (long long)nt_out * ntr;
    if (n > 0) k_akima<<<grid_for(n), 256, 0, st>>>(din, nt_in, dt_in, dout, nt_out, dt_out, ntr);
    PCK(cudaGetLastError());
    return FWI_OK;
}

}  // namespace fwi

using namespace fwi;

extern "C" {

int fwi_set_filter_order(int order) {
    if (order < 1 || order > 32) return prep_fail(FWI_ERR_ARG, "filter order must be in 1..32");
    std::lock_guard<std::mutex> g(PS().mu);
    PS().order = order;
    return FWI_OK;
}

int fwi_time_filter(float* Data_trace, const int* nt_, const float* dt_, const int* Num_, const int* typef_,
                    const float* f1_, const float* fc_) {
    PTRY(prep_ensure_init());
    if (!Data_trace || !nt_ || !dt_ || !Num_ || !typef_ || !f1_ || !fc_) return prep_fail(FWI_ERR_ARG, "null argument");
    const int nt = *nt_, Num = *Num_, typef = *typef_;
    const float dt = *dt_, f1 = *f1_, fc = *fc_;
    if (nt < 1 || Num < 0) return prep_fail(FWI_ERR_ARG, "nt must be >= 1 and Num >= 0");
    if (!(dt > 0.f)) return prep_fail(FWI_ERR_ARG, "dt must be positive");
    if (typef < 1 || typef > 3) return prep_fail(FWI_ERR_ARG, "typef must be 1 (low-pass), 2 (high-pass) or 3 (band-pass)");
    if (Num == 0) return FWI_OK;
    std::lock_guard<std::mutex> g(PS().mu);
    PrepState& S = PS();
    cudaStream_t st = prep_stream();
    const size_t bytes = (size_t)nt * Num * 4;
    const bool dev = prep_is_device_ptr(Data_trace);
    float* d = Data_trace;
    if (!dev) {
        PTRY(S.traces.ensure(bytes));
        d = reinterpret_cast<float*>(S.traces.p);
        PCK(cudaMemcpyAsync(d, Data_trace, bytes, cudaMemcpyHostToDevice, st));
    }
    PTRY(filter_traces_device(d, nt, dt, Num, typef, f1, fc));
    if (!dev) PCK(cudaMemcpyAsync(Data_trace, d, bytes, cudaMemcpyDeviceToHost, st));
    PCK(cudaStreamSynchronize(st));
    return FWI_OK;
}

int fwi_interpolation_akima(const float* Data_tmp, const float* dt_Data_, const int* nt_Data_, float* Data_trace,
                            const int* NumRec_, const float* dt_, const int* nt_) {
    PTRY(prep_ensure_init());
    if (!Data_tmp || !dt_Data_ || !nt_Data_ || !Data_trace || !NumRec_ || !dt_ || !nt_)
        return prep_fail(FWI_ERR_ARG, "null argument");
    const int nt_in = *nt_Data_, ntr = *NumRec_, nt_out = *nt_;
    const float dt_in = *dt_Data_, dt_out = *dt_;
    // INTRPL's error exits: fewer than 2 input points, no output point,
    // abscissae not increasing (akima433.f90:58-62, :160-168)
    if (nt_in < 2) return prep_fail(FWI_ERR_ARG, "nt_Data must be >= 2");
    if (nt_out < 1) return prep_fail(FWI_ERR_ARG, "nt must be >= 1");
    if (!(dt_in > 0.f) || !(dt_out > 0.f)) return prep_fail(FWI_ERR_ARG, "time steps must be positive");
    if (ntr < 0) return prep_fail(FWI_ERR_ARG, "NumRec must be >= 0");
    if (ntr == 0) return FWI_OK;
    std::lock_guard<std::mutex> g(PS().mu);
    PrepState& S = PS();
    cudaStream_t st = prep_stream();
    const size_t bin = (size_t)nt_in * ntr * 4, bout = (size_t)nt_out * ntr * 4;
    const bool din = prep_is_device_ptr(Data_tmp), dout = prep_is_device_ptr(Data_trace);
    const float* src = Data_tmp;
    float* dst = Data_trace;
    if (!din) {
        PTRY(S.traces.ensure(bin));
        PCK(cudaMemcpyAsync(S.traces.p, Data_tmp, bin, cudaMemcpyHostToDevice, st));
        src = reinterpret_cast<const float*>(S.traces.p);
    }
    if (!dout) {
        PTRY(S.out.ensure(bout));
        dst = reinterpret_cast<float*>(S.out.p);
    }
    PTRY(akima_device(src, nt_in, dt_in, dst, nt_out, dt_out, ntr));
    if (!dout) PCK(cudaMemcpyAsync(Data_trace, dst, bout, cudaMemcpyDeviceToHost, st));
    PCK(cudaStreamSynchronize(st));
    return FWI_OK;
}

// The WAS geometry of get_was_data.f90 (host arithmetic in the reference's
// FP32 operations and order; added_space_model = 0, modules.f90:153):
//   shots (the receivers of the reciprocal inversion): grid column
//     1+ceiling((0+|xs|)/dmodel)                                   :155-156
//   OBS (its sources): grid column 1+ceiling((0+|x|)/dmodel), depth |z| :201-205
//   bathymetry model: Akima's interpolation (INTRPL) through (0, shot
//     positions, length_model) and the shots' water depths (|bat|, the first
//     and last repeated at the ends) at (i-1)*dmodel, i = 1..nxmodel, with
//     length_model = (nxmodel-1)*dmodel (modules.f90:431)            :584-613
//   relocation: each OBS depth replaced by the model bathymetry at its
//     column, then its grid row 1+ceiling(z/dmodel)                   :112-115
//   indices: nxSou/nySou = the OBS column/row, nxRec = the shot columns,
//     nyRec = 1+ceiling(shot_depth/dmodel)                            :223-231
int fwi_was_geometry(int num_obs, const float* xobs, const float* zobs, int num_shots, const float* xshot,
                     const float* bat, float shot_depth, float dmodel, int nxmodel, int relocate, int* nxSou,
                     int* nySou, int* nxRec, int* nyRec, float* bat_model, int* bat_model_grid) {
    if (num_obs < 0 || num_shots < 0 || !(dmodel > 0.f)) return prep_fail(FWI_ERR_ARG, "bad WAS geometry sizes");
    if ((num_obs && (!xobs || !zobs)) || (num_shots && !xshot)) return prep_fail(FWI_ERR_ARG, "null argument");
    const bool need_model = relocate || bat_model || bat_model_grid;
    if (need_model && (num_shots < 1 || !bat || nxmodel < 1))
        return prep_fail(FWI_ERR_ARG, "the bathymetry model needs the shots' water depths and nxmodel >= 1");
    const float added_space_model = 0.f;
    std::vector<float> pos_shot(num_shots), pos_bat(num_shots);
    for (int i = 0; i < num_shots; ++i) {
        pos_shot[i] = added_space_model + fabsf(xshot[i]);
        if (nxRec) nxRec[i] = 1 + (int)ceilf(pos_shot[i] / dmodel);
        if (bat) pos_bat[i] = fabsf(bat[i]);
    }
    if (nyRec) *nyRec = 1 + (int)ceilf(shot_depth / dmodel);
    std::vector<float> model;
    if (need_model) {
        const int L = num_shots + 2;
        std::vector<float> xm(L), yb(L);
        for (int i = 2; i <= num_shots + 1; ++i) {
            yb[i - 1] = pos_bat[i - 2];
            xm[i - 1] = pos_shot[i - 2];
        }
        const float length_model = (float)(nxmodel - 1) * dmodel;
        xm[0] = 0.f;
        xm[L - 1] = length_model;
        yb[0] = yb[1];
        yb[L - 1] = yb[L - 2];
        for (int i = 1; i < L; ++i)  // INTRPL's check: abscissae increasing (akima433.f90:160-168)
            if (!(xm[i] > xm[i - 1]))
                return prep_fail(FWI_ERR_ARG, "shot positions must increase inside (0, (nxmodel-1)*dmodel)");
        model.resize(nxmodel);
        for (int i = 1; i <= nxmodel; ++i) {
            const float u = (float)(i - 1) * dmodel;
            model[i - 1] = akima_eval(yb.data(), L, ArrayAxis{xm.data()}, u);
            if (bat_model) bat_model[i - 1] = model[i - 1];
            if (bat_model_grid) bat_model_grid[i - 1] = 1 + (int)ceilf(model[i - 1] / dmodel);
        }
    }
    for (int i = 0; i < num_obs; ++i) {
        const float px = added_space_model + fabsf(xobs[i]);
        const int gx = 1 + (int)ceilf(px / dmodel);
        float pz = fabsf(zobs[i]);
        if (relocate) {
            if (gx < 1 || gx > nxmodel) return prep_fail(FWI_ERR_ARG, "OBS outside the bathymetry model");
            pz = model[gx - 1];
        }
        if (nxSou) nxSou[i] = gx;
        if (nySou) nySou[i] = 1 + (int)ceilf(pz / dmodel);
    }
    return FWI_OK;
}

}  // extern "C"
