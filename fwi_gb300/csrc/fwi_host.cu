// Host side of the FWI path: the C ABI declared in include/fwi_gb300.h.
//
// Responsibilities: argument validation (everything the reference would
// index out of bounds is rejected before launch), device layout planning,
// per-warp work lists with their source/receiver cells, the time-step
// schedule (snapshot counter of solver_acoustic_SS.f90:303-305, :438-471),
// wave sizing against the HBM budget, CUDA-graph capture of whole waves,
// and the misfit/gradient reductions of calculate_misfit_gradient.f90.
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "fwi_gb300.h"
#include "fwi_internal.cuh"
#include "fwi_lists.h"

namespace fwi {
cudaError_t launch_step2(int acc, int mode, int var, const StepParams& pf, cudaStream_t st);
cudaError_t launch_step(int acc, int mode, int kstrip, const StepParams& pm, const StepParams& pb, cudaStream_t sm,
                        cudaStream_t sb, cudaStream_t ss);
cudaError_t launch_step_fused(int acc, int mode, int kstrip, const StepParams& pm, const StepParams& pb,
                              cudaStream_t st);
cudaError_t configure_step_kernels();
cudaError_t launch_build_c2(float* c2, int nyt, int pitch, int off, int dn, int ny, int nx, const float* src, int ldv,
                            int x0, int from_lambda, float dt2, float d2, cudaStream_t st);
cudaError_t launch_rec_last(float* rec, int nt, int nrec, cudaStream_t st);
cudaError_t launch_misfit(const float* synth, const float* obs, float* adj, double* mis_tr, int nt, float dt,
                          const int* tr_off, int ntr, int nshots, double* mis_shot, cudaStream_t st);
cudaError_t launch_stack(double* G, int ny, int nxm, const void* shots, int nshots, int form, cudaStream_t st);
size_t stack_shot_size();
void fill_stack_shot(void* dst, const float* k32, const double* k64, int x0, int nx, int off_dn, int pitch, double w);
cudaError_t launch_finalize(float* grad, const double* G, int ny, int nxm, int numtasks, const int* water,
                            cudaStream_t st);
cudaError_t launch_fields_io(float* fort, float* snaps, int ny, int nx, int pitch, int off_dn, int nsnap, int to_dev,
                             cudaStream_t st);
cudaError_t launch_kernel_io(float* dev, float* fort, int ny, int nx, int pitch, int off_dn, int to_dev,
                             cudaStream_t st);
cudaError_t launch_dot(const float* g, const float* o, size_t n, double* part, int nb, double* out, cudaStream_t st);
cudaError_t launch_nonfinite(const float* a, size_t n, int* flag, cudaStream_t st);
cudaError_t launch_search_max(const float* search, const float* var, size_t n, unsigned* out, cudaStream_t st);
cudaError_t launch_model_update(const float* search, const float* var, float step, size_t n, float* lam,
                                cudaStream_t st);
size_t copy_job_size();
void fill_copy_job(void* dst, const void* src, void* to, size_t bytes);
cudaError_t launch_copy_jobs(const void* jobs, int njobs, cudaStream_t st);
}  // namespace fwi

using namespace fwi;

namespace {

// ---------------------------------------------------------------------------
// errors and library state
// ---------------------------------------------------------------------------

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}
int cuda_fail(cudaError_t e, const char* what, int line) {
    char buf[512];
    snprintf(buf, sizeof buf, "CUDA error %s (%s) in %s [fwi_host.cu:%d]", cudaGetErrorName(e), cudaGetErrorString(e),
             what, line);
    g_err = buf;
    return (e == cudaErrorMemoryAllocation) ? FWI_ERR_NOMEM : FWI_ERR_CUDA;
}
#define CK(x)                                                       \
    do {                                                            \
        cudaError_t e_ = (x);                                       \
        if (e_ != cudaSuccess) return cuda_fail(e_, #x, __LINE__);  \
    } while (0)
// launch + count (each launcher issues the number of kernels it returns in nk)
#define LK(x)                                                      \
    do {                                                           \
        cudaError_t e_ = (x);                                      \
        if (e_ != cudaSuccess) return cuda_fail(e_, #x, __LINE__); \
        ++L().launches;                                            \
    } while (0)
#define TRY(x)                  \
    do {                        \
        int r_ = (x);           \
        if (r_ != FWI_OK) return r_; \
    } while (0)

struct LibState {
    bool init = false;
    int device = 0;
    cudaStream_t own = nullptr;
    cudaStream_t user = nullptr;
    cudaStream_t aux = nullptr;      // bottom-row kernels run here, concurrently
    cudaStream_t aux3 = nullptr;     // side-strip kernels run here, concurrently
    cudaStream_t copy_in = nullptr;  // the batch call's observed-data uploads, beside the forward pass
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_join2 = nullptr;
    cudaEvent_t ev2[10] = {};  // two-step pipeline (two sets of five)
    int prio_hi = 0;
    int acc = 3, dpml = 20;
    // two-step kernel and tile height of the drop-in solver: the choice of
    // the last survey tuned in this process (the tuner's default before)
    int tile_var = 1, tile_band = TWO_STEP_BAND, tile_eband = 0;
    long long launches = 0;
    std::recursive_mutex mu;
};
LibState& L() {
    static LibState s;
    return s;
}
cudaStream_t stream() { return L().user ? L().user : L().own; }

// Every entry point works on the library's device: it is made current on the
// calling thread (a caller that switched devices, or another host thread,
// would otherwise launch on a device that does not own the library's streams).
int ensure_init() {
    if (!L().init) return fwi_init(0);
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess || cur != L().device) CK(cudaSetDevice(L().device));
    return FWI_OK;
}

// device allocation with RAII
struct DBuf {
    void* p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    int alloc(size_t bytes) {
        release();
        if (bytes == 0) bytes = 16;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) {
            p = nullptr;
            char buf[256];
            snprintf(buf, sizeof buf, "cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
            g_err = buf;
            return FWI_ERR_NOMEM;
        }
        n = bytes;
        return FWI_OK;
    }
    int ensure(size_t bytes) { return (p && n >= bytes) ? FWI_OK : alloc(bytes); }
    template <typename T> T* as() const { return reinterpret_cast<T*>(p); }
};

// ---------------------------------------------------------------------------
// coefficients (solver_FD_coeffs.f90, solver_PML_coeffs.f90); this file is
// built with -ffp-contract=off so the FP32 arithmetic matches the Fortran.
// ---------------------------------------------------------------------------

void fd_taps(int acc, float* c1, float* c2) {
    for (int i = 0; i <= MAXR; ++i) c1[i] = c2[i] = 0.f;
    if (acc == 3) {
        c1[0] = 0.f; c1[1] = 3.f / 4.f; c1[2] = -(3.f / 20.f); c1[3] = 1.f / 60.f;
        c2[0] = -(49.f / 18.f); c2[1] = 3.f / 2.f; c2[2] = -(3.f / 20.f); c2[3] = 1.f / 90.f;
    } else if (acc == 4) {
        c1[0] = 0.f; c1[1] = 4.f / 5.f; c1[2] = -(1.f / 5.f); c1[3] = 4.f / 105.f; c1[4] = -(1.f / 280.f);
        c2[0] = -(205.f / 72.f); c2[1] = 8.f / 5.f; c2[2] = -(1.f / 5.f); c2[3] = 8.f / 315.f; c2[4] = -(1.f / 560.f);
    }
    c2[0] = c2[0] / 2.f;  // centre tap halved (solver_FD_coeffs.f90:68)
}

// 1-D CPML factors A, B (0-based, dn entries; entries 0..acc-1 are zero).
// The corner matrices of the reference are A(max(i,j)) in the orientation
// of each corner and are indexed on the fly by the kernels.
void pml_factors(int acc, int dpml, float dt, float d, std::vector<float>& fA, std::vector<float>& fB) {
    const int dn = dpml + 2 * acc;
    fA.assign(dn, 0.f);
    fB.assign(dn, 0.f);
    const float pi = 3.14159265f, Refl = 0.00001f;
    const float wPML = (float)(dpml - 1) * d;
    const float lr = logf(Refl);
    for (int i = 1 + acc; i <= dpml + acc; ++i) {
        const float y = (float)(i - (acc + 1)) * d;
        const float q = y / wPML;
        const float alpha = 30.f * pi * (1.f - (y / wPML));
        const float sigma = (-((6000.f * lr) / (2.f * wPML))) * (q * q);
        const float A = expf((-(sigma + alpha)) * dt);
        fA[i - 1] = A;
        fB[i - 1] = ((A - 1.f) * sigma) / (sigma + alpha);
    }
    for (int i = dpml + acc + 1; i <= dn; ++i) {
        fA[i - 1] = fA[dpml + acc - 1];
        fB[i - 1] = fB[dpml + acc - 1];
    }
}

// layout and work lists: fwi_lists.cpp

int validate_common(int ny, int nx, int acc, int dpml, int nt, int store_snap) {
    if (acc != 3 && acc != 4) return fail(FWI_ERR_ARG, "acc must be 3 or 4 (the reference's 6th/8th-order tables)");
    if (dpml < 1 || dpml + 2 * acc > MAXDN - 2)
        return fail(FWI_ERR_ARG, "dpml must be >= 1 and dpml + 2*acc <= 62");
    if (ny < 1 || nx < 1) return fail(FWI_ERR_ARG, "ny and nx must be >= 1");
    if ((long long)ny * nx > (1LL << 31)) return fail(FWI_ERR_ARG, "model too large");
    if (nt < 2) return fail(FWI_ERR_ARG, "nt must be >= 2");
    if (store_snap < 1) return fail(FWI_ERR_ARG, "store_snap must be >= 1");
    return FWI_OK;
}

int validate_geometry(const ShotGeom& g, const Layout& l, int shot) {
    char buf[256];
    auto chk = [&](const std::vector<int>& xs, const std::vector<int>& ys, const char* what) -> int {
        for (size_t i = 0; i < xs.size(); ++i) {
            const int py = l.dn + ys[i], px = l.dn + xs[i];
            if (py < 1 || py > l.nyt || px < 1 || px > l.nxt) {
                snprintf(buf, sizeof buf,
                         "shot %d: %s %zu at grid (%d,%d) lies outside the padded grid (rows 1..%d, cols 1..%d "
                         "after padding by %d)",
                         shot, what, i + 1, ys[i], xs[i], l.nyt, l.nxt, l.dn);
                return fail(FWI_ERR_ARG, buf);
            }
        }
        return FWI_OK;
    };
    TRY(chk(g.nxS, g.nyS, "source"));
    TRY(chk(g.nxR, g.nyR, "receiver"));
    return FWI_OK;
}

template <typename T>
int upload(DBuf& b, const std::vector<T>& v, cudaStream_t st) {
    TRY(b.ensure(std::max<size_t>(v.size() * sizeof(T), 16)));
    if (!v.empty()) CK(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    return FWI_OK;
}

bool is_device_ptr(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

double step_bytes_shot(int ny, int nx, int dn) {
    const double cells = (double)(ny + dn) * (double)(nx + 2 * dn);
    const double cpml = 2.0 * ny * dn + (double)dn * nx + 4.0 * dn * dn;
    return 16.0 * cells + 16.0 * cpml;
}

// ---------------------------------------------------------------------------
// per-shot device state
// ---------------------------------------------------------------------------

struct ShotState {
    DBuf pa, pb, pc, pd, c2, phx, chx, phy, phy2, chy, snaps, sscale, k;  // pc, pd: second wavefield pair
    DBuf bst[9];   // second state (adjoint) when recomputing: the seven fields, then its second wavefield pair
    DBuf ckpt;     // forward-state checkpoints when recomputing
    Layout lay{};
    size_t field_bytes = 0, snap_bytes = 0;
    // the seven fields of a checkpointed state (the state is in wavefield pair 0
    // at every checkpoint): pa, pb, phx, chx, phy, phy2, chy
    void* state(int i) {
        DBuf* a[7] = {&pa, &pb, &phx, &chx, &phy, &phy2, &chy};
        return a[i]->p;
    }
    size_t bytes() const {
        size_t n = pa.n + pb.n + pc.n + pd.n + c2.n + phx.n + chx.n + phy.n + phy2.n + chy.n + snaps.n + sscale.n + k.n + ckpt.n;
        for (auto& b : bst) n += b.n;
        return n;
    }
    int alloc_rc(int nckpt) {
        for (auto& b : bst) TRY(b.ensure(field_bytes));
        TRY(ckpt.ensure(std::max<size_t>(16, (size_t)nckpt * 7 * field_bytes)));
        return FWI_OK;
    }
    int alloc(const Layout& l, int nsnap_blocks, int snap_form, int grad_form) {
        lay = l;
        field_bytes = (size_t)l.nyt * l.pitch * sizeof(float);
        const size_t esz = snap_form == FWI_SNAP_F32 ? 4 : 2;
        snap_bytes = (size_t)nsnap_blocks * l.ny * l.pitch * esz;
        TRY(pa.ensure(field_bytes));
        TRY(pb.ensure(field_bytes));
        TRY(pc.ensure(field_bytes));
        TRY(pd.ensure(field_bytes));
        TRY(c2.ensure(field_bytes));
        TRY(phx.ensure(field_bytes));
        TRY(chx.ensure(field_bytes));
        TRY(phy.ensure(field_bytes));
        TRY(phy2.ensure(field_bytes));
        TRY(chy.ensure(field_bytes));
        TRY(snaps.ensure(snap_bytes));
        TRY(sscale.ensure((size_t)nsnap_blocks * l.ny * (l.ntiles + 2) * sizeof(float)));
        TRY(k.ensure((size_t)l.ny * l.pitch * (grad_form == FWI_GRAD_F64 ? 8 : 4)));
        return FWI_OK;
    }
    int zero_state(cudaStream_t st) {
        CK(cudaMemsetAsync(pa.p, 0, field_bytes, st));
        CK(cudaMemsetAsync(pb.p, 0, field_bytes, st));
        CK(cudaMemsetAsync(pc.p, 0, field_bytes, st));
        CK(cudaMemsetAsync(pd.p, 0, field_bytes, st));
        CK(cudaMemsetAsync(phx.p, 0, field_bytes, st));
        CK(cudaMemsetAsync(chx.p, 0, field_bytes, st));
        CK(cudaMemsetAsync(phy.p, 0, field_bytes, st));
        CK(cudaMemsetAsync(phy2.p, 0, field_bytes, st));
        CK(cudaMemsetAsync(chy.p, 0, field_bytes, st));
        return FWI_OK;
    }
    ShotDev dev(int nt, int nrec, int x0, const float* srcv, float* rec) const {
        ShotDev d{};
        d.pf[0] = pa.as<float>();
        d.pf[1] = pb.as<float>();
        d.pf[2] = pc.as<float>();
        d.pf[3] = pd.as<float>();
        d.c2 = c2.as<float>();
        d.phx = phx.as<float>();
        d.chx = chx.as<float>();
        d.phy = phy.as<float>();
        d.phy2 = phy2.as<float>();
        d.chy = chy.as<float>();
        d.srcv = srcv;
        d.rec = rec;
        d.snaps = snaps.p;
        d.sscale = sscale.as<float>();
        d.k32 = k.as<float>();
        d.k64 = k.as<double>();
        d.snap_stride = (long long)lay.ny * lay.pitch;
        d.ny = lay.ny;
        d.nx = lay.nx;
        d.nyt = lay.nyt;
        d.nxt = lay.nxt;
        d.off = lay.off;
        d.pitch = lay.pitch;
        d.ntiles = lay.ntiles;
        d.dn = lay.dn;
        d.sl = lay.sl;
        d.sr = lay.sr;
        d.nt = nt;
        d.nrec = nrec;
        d.x0 = x0;
        return d;
    }
};

StepParams base_params(int acc, float dt, int store_snap, int snap_form, int grad_form, const float* dfA,
                       const float* dfB) {
    StepParams p{};
    float c1[MAXR + 1], c2[MAXR + 1];
    fd_taps(acc, c1, c2);
    for (int i = 0; i <= MAXR; ++i) {
        p.c1[i] = c1[i];
        p.c2[i] = c2[i];
    }
    p.fA = dfA;
    p.fB = dfB;
    p.dt = dt;
    // RN(1/dt) for the snapshot quotient (fwi_div.cuh); a dt whose reciprocal
    // is not a normal float falls back to the division
    p.rdt = (dt >= 0x1p-60f && dt <= 0x1p60f) ? 1.f / dt : 0.f;
    p.ss = (float)store_snap;
    p.snap_form = snap_form;
    p.grad_form = grad_form;
    p.snap = -1;
    return p;
}

struct StepSet {
    StepParams pm, pb;  // interior list; boundary list (pb.nstrip side strips, then bottom tiles)
    int kstrip = 1;
    bool fused = false;  // single steps as one launch (k_step_fused) instead of three on three streams
};

// Wavefield buffers of step k.  A shot's state (p, p_1) lives in pair 0
// (pf[0], pf[1]) or pair 1 (pf[2], pf[3]); within a pair, step k reads p from
// the first buffer for odd k and from the second for even k, and writes p_3
// over p_1 (the reference's two-array rotation of p and p_1).
inline int cur_buf(int k, int pair) { return 2 * pair + ((k & 1) ? 0 : 1); }
inline int prev_buf(int k, int pair) { return 2 * pair + ((k & 1) ? 1 : 0); }

// Parameters of the single step k with the state in `pair` (sn: snapshot
// block or -1).
void set_step(StepSet& ps, int k, int sn, int pair = 0) {
    for (StepParams* p : {&ps.pm, &ps.pb}) {
        p->t = k - 2;
        p->parity = k & 1;
        p->snap = sn;
        p->rp = cur_buf(k, pair);
        p->rp1 = p->wo = p->wo2 = prev_buf(k, pair);
    }
}

// Two-step passes.  Steps k and k+1 run as: the single-step lists `lo` (the
// interior items outside the two-step tiles and the boundary list) for step
// k, concurrently with the two-step tiles `pf` (steps k and k+1), then `lo`
// for step k+1.  Inputs are read from the state pair X and both steps are
// written to the other pair Y, so no warp overwrites a p_n or p_{n-1} that a
// neighbour still reads; the state moves to pair Y (two_step_run).
struct TwoStep {
    StepParams pf;  // the first ncore items are core tiles
    StepSet lo;
    int ncore = 0;
    int var = 0;           // two-step kernel: 0 k_step2_interior, 1 k_step2s_interior
    bool snap_ok = false;  // a pass's first step may store a snapshot / image
};

// Two-step lists of a wave from its single-step set: the two-step tiles,
// and the single-step interior items outside them beside the boundary list.
TwoStep two_step_set(const StepSet& ps, int mode, const DBuf& fus, int nfus, int ncore, const DBuf& lft, int nlft,
                     int var) {
    TwoStep tw;
    tw.ncore = ncore;
    tw.var = var;
    tw.pf = ps.pm;
    tw.pf.items = fus.as<WorkItem>();
    tw.pf.nitems = nfus;
    tw.lo = ps;
    tw.lo.pm.items = lft.as<WorkItem>();
    tw.lo.pm.nitems = nlft;
    // the two-step kernel stores FP32 snapshots (a 16-bit snapshot's scale is
    // the maximum over a 128-column segment, which the single-step kernel
    // reduces within one warp) and images with any form
    tw.snap_ok = mode == 1 || ps.pm.snap_form == FWI_SNAP_F32;
    return tw;
}

int step_kernels(const StepSet& ps) {
    return (ps.pm.nitems > 0) + (ps.pb.nstrip > 0) + (ps.pb.nitems > ps.pb.nstrip);
}

// One time step: interior tiles on st, bottom tiles on st2, side strips on
// the library's third stream, all three ordered after the previous step and
// before the next one.  Streams fork only when st itself gets a kernel (a
// wait on an event with no new node on st in between would accumulate
// dependencies under stream capture).
int step_fork_join(int acc, int mode, const StepSet& ps, cudaStream_t st, cudaStream_t st2) {
    const bool has_m = ps.pm.nitems > 0, has_b = ps.pb.nitems > ps.pb.nstrip, has_s = ps.pb.nstrip > 0;
    if (ps.fused) {
        L().launches += (has_m || has_b || has_s) ? 1 : 0;
        CK(launch_step_fused(acc, mode, ps.kstrip, ps.pm, ps.pb, st));
        return FWI_OK;
    }
    L().launches += step_kernels(ps);
    if (!has_m || (!has_s && !has_b)) {
        CK(launch_step(acc, mode, ps.kstrip, ps.pm, ps.pb, st, st, st));
        return FWI_OK;
    }
    cudaStream_t st3 = L().aux3;
    CK(cudaEventRecord(L().ev_fork, st));
    if (has_b) CK(cudaStreamWaitEvent(st2, L().ev_fork, 0));
    if (has_s) CK(cudaStreamWaitEvent(st3, L().ev_fork, 0));
    CK(launch_step(acc, mode, ps.kstrip, ps.pm, ps.pb, st, st2, st3));
    if (has_b) {
        CK(cudaEventRecord(L().ev_join, st2));
        CK(cudaStreamWaitEvent(st, L().ev_join, 0));
    }
    if (has_s) {
        CK(cudaEventRecord(L().ev_join2, st3));
        CK(cudaStreamWaitEvent(st, L().ev_join2, 0));
    }
    return FWI_OK;
}

// npass consecutive two-step passes from step k, state in pair X.  Pass j
// (steps k, k+1; inputs in pair X, outputs in pair Y) is
//   C(j)  the core tiles (both steps), on st;
//   E(j)  the edge tiles (both steps), on st2;
//   A(j)  step k of the single-step lists: interior items and bottom tiles
//         on st2 (A2), side strips on aux3 (A3);
//   B(j)  step k+1 of the single-step lists (B2 on st2, B3 on aux3).
// Core tiles read only two-step cells and the top pad; the cells next to the
// single-step cells belong to edge tiles.  So
//   C(j) waits for C(j-1) and E(j-1);  E(j) for C(j-1) and B(j-1);
//   A(j) for B(j-1) and E(j-1);        B(j) for A(j) and E(j),
// and the single-step chain A, B runs beside the core tiles.  Kernels in
// flight together never write a cell another one reads: every kernel writes
// only its own cells, the tiles write pair Y while the core tiles of the next
// pass read it only where the finished tiles wrote, and the single-step
// kernels read the pair they do not write only at their own cells.
// sn[j]: snapshot block that pass j's first step stores / images with (-1: none).
int two_step_run(int acc, int mode, const TwoStep& tw, int k, int npass, const int* sn, int X, cudaStream_t st,
                 cudaStream_t st2) {
    cudaStream_t st3 = L().aux3;
    cudaEvent_t* ev = L().ev2;  // [set][C, E, A3, B2, B3]
    auto C = [&](int p) { return ev[5 * p + 0]; };
    auto E = [&](int p) { return ev[5 * p + 1]; };
    auto A3 = [&](int p) { return ev[5 * p + 2]; };
    auto B2 = [&](int p) { return ev[5 * p + 3]; };
    auto B3 = [&](int p) { return ev[5 * p + 4]; };
    // entry: everything so far is on st; set 1 stands for "pass -1"
    CK(cudaEventRecord(C(1), st));
    CK(cudaEventRecord(E(1), st));
    CK(cudaStreamWaitEvent(st2, C(1), 0));
    CK(cudaStreamWaitEvent(st3, C(1), 0));
    CK(cudaEventRecord(B2(1), st2));
    CK(cudaEventRecord(B3(1), st3));
    StepParams fc = tw.pf, fe = tw.pf;
    fc.nitems = tw.ncore;
    fe.items = tw.pf.items + tw.ncore;
    fe.nitems = tw.pf.nitems - tw.ncore;
    int p = 0;
    for (int j = 0; j < npass; ++j, k += 2, X ^= 1, p ^= 1) {
        const int Y = X ^ 1, q = p ^ 1;
        StepSet a = tw.lo, b = tw.lo;
        for (StepParams* sp : {&a.pm, &a.pb, &fc, &fe}) {
            sp->t = k - 2;
            sp->parity = k & 1;
            sp->snap = sn ? sn[j] : -1;
            sp->rp = cur_buf(k, X);
            sp->rp1 = prev_buf(k, X);
            sp->wo = sp->wo2 = prev_buf(k, Y);
        }
        fc.wo2 = fe.wo2 = prev_buf(k + 1, Y);
        for (StepParams* sp : {&b.pm, &b.pb}) {
            sp->t = k - 1;
            sp->parity = (k + 1) & 1;
            sp->snap = -1;
            sp->rp = cur_buf(k + 1, Y);  // step k's output
            sp->rp1 = cur_buf(k, X);     // p_n
            sp->wo = sp->wo2 = prev_buf(k + 1, Y);
        }
        StepSet a2 = a, a3 = a, b2 = b, b3 = b;  // the st2 part (no strips) and the strip part
        a2.pb.nstrip = b2.pb.nstrip = 0;
        a2.pb.items = a.pb.items + a.pb.nstrip;
        a2.pb.nitems = a.pb.nitems - a.pb.nstrip;
        b2.pb.items = a2.pb.items;
        b2.pb.nitems = a2.pb.nitems;
        a3.pm.nitems = b3.pm.nitems = 0;
        a3.pb.nitems = b3.pb.nitems = a.pb.nstrip;
        L().launches += 2 * step_kernels(a) + (fc.nitems > 0) + (fe.nitems > 0);
        // C(j)
        CK(cudaStreamWaitEvent(st, E(q), 0));
        CK(launch_step2(acc, mode, tw.var, fc, st));
        CK(cudaEventRecord(C(p), st));
        // A3(j)
        CK(cudaStreamWaitEvent(st3, B2(q), 0));
        CK(launch_step(acc, mode, a3.kstrip, a3.pm, a3.pb, st3, st3, st3));
        CK(cudaEventRecord(A3(p), st3));
        // A2(j), then E(j)
        CK(cudaStreamWaitEvent(st2, B3(q), 0));
        CK(launch_step(acc, mode, a2.kstrip, a2.pm, a2.pb, st2, st2, st2));
        CK(cudaStreamWaitEvent(st2, C(q), 0));
        CK(launch_step2(acc, mode, tw.var, fe, st2));
        CK(cudaEventRecord(E(p), st2));
        // B3(j) after A2(j) and E(j); B2(j) after A3(j)
        CK(cudaStreamWaitEvent(st3, E(p), 0));
        CK(launch_step(acc, mode, b3.kstrip, b3.pm, b3.pb, st3, st3, st3));
        CK(cudaEventRecord(B3(p), st3));
        CK(cudaStreamWaitEvent(st2, A3(p), 0));
        CK(launch_step(acc, mode, b2.kstrip, b2.pm, b2.pb, st2, st2, st2));
        CK(cudaEventRecord(B2(p), st2));
    }
    // exit: everything joins st
    CK(cudaStreamWaitEvent(st, B2(p ^ 1), 0));
    CK(cudaStreamWaitEvent(st, B3(p ^ 1), 0));
    return FWI_OK;
}

// Steps k0..k1; sn_of(k) is the snapshot block step k stores (forward) or
// images with (adjoint), -1 for none.  Pairs of steps run as two-step passes
// (when tw is given) where the second step has no snapshot and the first has
// none or tw allows it; the rest run as single steps.  The state is in pair 0
// before and after (an even number of passes).
template <typename SnOf>
int run_range(int acc, int mode, int k0, int k1, SnOf sn_of, StepSet& ps, const TwoStep* tw, cudaStream_t st,
              cudaStream_t st2) {
    if (k1 < k0) return FWI_OK;
    std::vector<int> sn(k1 + 2, -1);
    for (int k = k0; k <= k1; ++k) sn[k] = sn_of(k);
    const std::vector<StepUnit> units = plan_steps(k0, k1, sn, tw != nullptr, tw && tw->snap_ok);
    int pair = 0;
    std::vector<int> sns;
    for (size_t i = 0; i < units.size();) {
        if (units[i].pass) {
            size_t j = i;
            sns.clear();
            while (j < units.size() && units[j].pass) sns.push_back(units[j++].sn);
            TRY(two_step_run(acc, mode, *tw, units[i].k, (int)sns.size(), sns.data(), pair, st, st2));
            pair ^= (int)(sns.size() & 1);
            i = j;
            continue;
        }
        set_step(ps, units[i].k, units[i].sn, pair);
        TRY(step_fork_join(acc, mode, ps, st, st2));
        ++i;
    }
    return FWI_OK;
}

// One pass over the time loop k = 2..nt for a set of shots.
// mode 0: forward (snapshots if store, receivers recorded); mode 1: adjoint.
// tw: two-step passes (null: single steps only).
int run_time_loop(int acc, int mode, int nt, int store_snap, int nt_store, bool store, StepSet ps, cudaStream_t st,
                  cudaStream_t st2, const TwoStep* tw = nullptr) {
    const std::vector<int> ev = snapshot_steps(nt, store_snap);
    std::vector<int> sn(nt + 2, -1);
    int snap = (mode == 0) ? 0 : nt_store;
    for (int e : ev) {
        if (mode == 0) {
            ++snap;
            sn[e] = store ? snap : -1;
        } else {
            --snap;
            sn[e] = snap;
        }
    }
    return run_range(acc, mode, 2, nt, [&](int k) { return sn[k]; }, ps, tw, st, st2);
}

// ---------------------------------------------------------------------------
// single-shot drop-in state (buffers kept between calls)
// ---------------------------------------------------------------------------

struct Single {
    ShotState sh;
    DBuf d_ctmp, d_srcv, d_rec, d_items_m, d_items_b, d_src, d_recs, d_shot, d_fA, d_fB, d_stage, d_flag;
    DBuf d_items_f, d_items_l;  // two-step tiles; single-step interior items beside them
};
Single& single() {
    static Single s;
    return s;
}

// The plan of fwi_misfit_gradient_batch: the survey of the last geometry seen
// (one survey: a new geometry frees the previous one's device memory before
// it plans, so the wave sizes always see the whole device).
struct BatchPlan {
    std::string key;
    fwi_survey* s = nullptr;
    long long plans = 0;
    void release() {
        if (s) fwi_survey_destroy(s);
        s = nullptr;
        key.clear();
    }
};
BatchPlan& batch_plan() {
    static BatchPlan b;
    return b;
}

int check_nonfinite(const float* dptr, size_t n, DBuf& flag, cudaStream_t st, const char* what) {
    TRY(flag.ensure(sizeof(int)));
    CK(cudaMemsetAsync(flag.p, 0, sizeof(int), st));
    LK(launch_nonfinite(dptr, n, flag.as<int>(), st));
    int h = 0;
    CK(cudaMemcpyAsync(&h, flag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (h) return fail(FWI_ERR_NONFINITE, std::string("non-finite values in ") + what +
                                              " (the time step may violate the CFL limit)");
    return FWI_OK;
}

}  // namespace

// Library services for the pre-processing entry points (fwi_prep.cu).
namespace fwi {
int prep_fail(int code, const std::string& msg) { return fail(code, msg); }
cudaStream_t prep_stream() { return stream(); }
bool prep_is_device_ptr(const void* p) { return is_device_ptr(p); }
int prep_ensure_init() {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    return ensure_init();
}
}  // namespace fwi

// ===========================================================================
// C ABI
// ===========================================================================

extern "C" {

int fwi_init(int device) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    if (L().init && L().device == device) {
        CK(cudaSetDevice(device));
        return FWI_OK;
    }
    int n = 0;
    CK(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return fail(FWI_ERR_ARG, "invalid CUDA device index");
    // a new device: the streams, events and buffers of the old one are released
    if (L().init) TRY(fwi_finalize());
    CK(cudaSetDevice(device));
    if (!L().own) CK(cudaStreamCreateWithFlags(&L().own, cudaStreamNonBlocking));
    if (!L().aux) {
        // boundary kernels (long dependency chains, few warps) get the
        // higher priority so they start first and overlap the interior
        int lo = 0, hi = 0;
        CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        CK(cudaStreamCreateWithPriority(&L().aux, cudaStreamNonBlocking, hi));
        L().prio_hi = hi;
    }
    if (!L().aux3) {
        int lo = 0, hi = 0;
        CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        CK(cudaStreamCreateWithPriority(&L().aux3, cudaStreamNonBlocking, hi));
    }
    if (!L().copy_in) CK(cudaStreamCreateWithFlags(&L().copy_in, cudaStreamNonBlocking));
    if (!L().ev_fork) CK(cudaEventCreateWithFlags(&L().ev_fork, cudaEventDisableTiming));
    if (!L().ev_join) CK(cudaEventCreateWithFlags(&L().ev_join, cudaEventDisableTiming));
    if (!L().ev_join2) CK(cudaEventCreateWithFlags(&L().ev_join2, cudaEventDisableTiming));
    for (auto& e : L().ev2)
        if (!e) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    CK(configure_step_kernels());
    L().device = device;
    L().init = true;
    return FWI_OK;
}

int fwi_finalize(void) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    if (!L().init) return FWI_OK;
    cudaDeviceSynchronize();
    batch_plan().release();
    Single& s = single();
    s.~Single();
    new (&s) Single();
    if (L().own) cudaStreamDestroy(L().own);
    if (L().aux) cudaStreamDestroy(L().aux);
    if (L().aux3) cudaStreamDestroy(L().aux3);
    if (L().copy_in) cudaStreamDestroy(L().copy_in);
    if (L().ev_fork) cudaEventDestroy(L().ev_fork);
    if (L().ev_join) cudaEventDestroy(L().ev_join);
    if (L().ev_join2) cudaEventDestroy(L().ev_join2);
    for (auto& e : L().ev2) {
        if (e) cudaEventDestroy(e);
        e = nullptr;
    }
    L().own = L().aux = L().aux3 = L().copy_in = nullptr;
    L().ev_fork = L().ev_join = L().ev_join2 = nullptr;
    L().user = nullptr;
    L().init = false;
    return FWI_OK;
}

const char* fwi_last_error(void) { return g_err.c_str(); }

int fwi_set_stream(void* st) {
    TRY(ensure_init());
    L().user = reinterpret_cast<cudaStream_t>(st);
    return FWI_OK;
}

int fwi_set_solver_options(int acc, int dpml) {
    if (acc != 3 && acc != 4) return fail(FWI_ERR_ARG, "acc must be 3 or 4");
    if (dpml < 1 || dpml + 2 * acc > MAXDN - 2) return fail(FWI_ERR_ARG, "dpml out of range");
    L().acc = acc;
    L().dpml = dpml;
    return FWI_OK;
}

int64_t fwi_kernel_launch_count(void) { return L().launches; }

int fwi_solver_acoustic_ss(const int* rank, const int* iprop_, const int* NumSou_, const int* NumRec_,
                           const int* nxSou, const int* nySou, const int* nxRec, const int* nyRec, const float* S,
                           const float* Sadj, const float* d_, const float* dt_, const int* ny_, const int* nx_,
                           const float* ctmp, const int* store_snap_, const int* nt_Store_, const int* nt_,
                           float* kernel, float* Fields, float* Rec_point) {
    (void)rank;
    std::lock_guard<std::recursive_mutex> g(L().mu);
    TRY(ensure_init());
    if (!iprop_ || !NumSou_ || !NumRec_ || !d_ || !dt_ || !ny_ || !nx_ || !store_snap_ || !nt_Store_ || !nt_)
        return fail(FWI_ERR_ARG, "null scalar argument");
    const int iprop = *iprop_, NumSou = *NumSou_, NumRec = *NumRec_, ny = *ny_, nx = *nx_;
    const int store_snap = *store_snap_, nt_store = *nt_Store_, nt = *nt_;
    const float d = *d_, dt = *dt_;
    const int acc = L().acc, dpml = L().dpml;
    TRY(validate_common(ny, nx, acc, dpml, nt, store_snap));
    if (NumSou < 0 || NumRec < 0) return fail(FWI_ERR_ARG, "NumSou/NumRec must be >= 0");
    if (!(d > 0.f) || !(dt > 0.f)) return fail(FWI_ERR_ARG, "d and dt must be positive");
    if (!ctmp || !Rec_point) return fail(FWI_ERR_ARG, "null ctmp or Rec_point");
    if (iprop == 2 && (!Sadj || !Fields || !kernel || !nxRec || !nyRec))
        return fail(FWI_ERR_ARG, "adjoint needs Sadj, Fields, kernel and receiver indices");
    if (iprop != 2 && NumSou > 0 && (!S || !nxSou || !nySou)) return fail(FWI_ERR_ARG, "forward needs S and sources");
    if (iprop == 1 && !Fields) return fail(FWI_ERR_ARG, "forward with iprop=1 needs Fields");
    if (NumRec > 0 && (!nxRec || !nyRec)) return fail(FWI_ERR_ARG, "null receiver indices");
    if (nt_store < 0) return fail(FWI_ERR_ARG, "nt_Store must be >= 0");
    const std::vector<int> ev = snapshot_steps(nt, store_snap);
    if ((iprop == 1 || iprop == 2) && (int)ev.size() > nt_store)
        return fail(FWI_ERR_ARG, "nt_Store is smaller than the number of snapshots nt/store_snap (the reference "
                                 "would write past Fields)");

    const Layout l = make_layout(ny, nx, acc, dpml);
    ShotGeom geo;
    geo.nx = nx;
    if (iprop != 2) {
        geo.nxS.assign(nxSou, nxSou + NumSou);
        geo.nyS.assign(nySou, nySou + NumSou);
    }
    if (NumRec > 0) {
        geo.nxR.assign(nxRec, nxRec + NumRec);
        geo.nyR.assign(nyRec, nyRec + NumRec);
    }
    TRY(validate_geometry(geo, l, 1));

    Single& sg = single();
    cudaStream_t st = stream();
    const int nsnap_blocks = nt_store + 1;
    TRY(sg.sh.alloc(l, (iprop == 1 || iprop == 2) ? nsnap_blocks : 1, FWI_SNAP_F32, FWI_GRAD_F32));
    TRY(sg.sh.zero_state(st));

    // model -> c2
    TRY(sg.d_ctmp.ensure((size_t)ny * nx * sizeof(float)));
    CK(cudaMemcpyAsync(sg.d_ctmp.p, ctmp, (size_t)ny * nx * sizeof(float), cudaMemcpyHostToDevice, st));
    LK(launch_build_c2(sg.sh.c2.as<float>(), l.nyt, l.pitch, l.off, l.dn, ny, nx, sg.d_ctmp.as<float>(), ny, 0, 0,
                       dt * dt, d * d, st));
    std::vector<float> fA, fB;
    pml_factors(acc, dpml, dt, d, fA, fB);
    TRY(upload(sg.d_fA, fA, st));
    TRY(upload(sg.d_fB, fB, st));

    // injected values
    const int nval = (iprop == 2) ? NumRec : NumSou;
    const float* hval = (iprop == 2) ? Sadj : S;
    TRY(sg.d_srcv.ensure(std::max<size_t>((size_t)nt * nval * sizeof(float), 16)));
    if (nval > 0) CK(cudaMemcpyAsync(sg.d_srcv.p, hval, (size_t)nt * nval * sizeof(float), cudaMemcpyHostToDevice, st));
    TRY(sg.d_rec.ensure(std::max<size_t>((size_t)nt * NumRec * sizeof(float), 16)));
    CK(cudaMemsetAsync(sg.d_rec.p, 0, std::max<size_t>((size_t)nt * NumRec * sizeof(float), 16), st));

    const int off_dn = l.off + l.dn;
    if (iprop == 2) {
        const size_t fbytes = (size_t)ny * nx * nsnap_blocks * sizeof(float);
        TRY(sg.d_stage.ensure(fbytes));
        CK(cudaMemcpyAsync(sg.d_stage.p, Fields, fbytes, cudaMemcpyHostToDevice, st));
        LK(launch_fields_io(sg.d_stage.as<float>(), sg.sh.snaps.as<float>(), ny, nx, l.pitch, off_dn, nsnap_blocks, 1,
                            st));
        CK(cudaMemsetAsync(sg.sh.k.p, 0, (size_t)ny * l.pitch * sizeof(float), st));
        TRY(sg.d_ctmp.ensure((size_t)ny * nx * sizeof(float)));
        CK(cudaMemcpyAsync(sg.d_ctmp.p, kernel, (size_t)ny * nx * sizeof(float), cudaMemcpyHostToDevice, st));
        LK(launch_kernel_io(sg.sh.k.as<float>(), sg.d_ctmp.as<float>(), ny, nx, l.pitch, off_dn, 1, st));
    }

    // work lists (the adjoint injects at the receivers)
    std::vector<ShotGeom> geoms{geo};
    std::vector<Layout> lays{l};
    Lists lists = build_lists(geoms, lays, 64, L().tile_band, L().tile_eband);
    const bool adj = (iprop == 2);
    TRY(upload(sg.d_items_m, adj ? lists.int_adj : lists.int_fwd, st));
    TRY(upload(sg.d_items_b, adj ? lists.bnd_adj : lists.bnd_fwd, st));
    TRY(upload(sg.d_items_f, adj ? lists.fus_adj : lists.fus_fwd, st));
    TRY(upload(sg.d_items_l, adj ? lists.lft_adj : lists.lft_fwd, st));
    TRY(upload(sg.d_src, adj ? lists.src_adj : lists.src_fwd, st));
    TRY(upload(sg.d_recs, lists.recs, st));
    std::vector<ShotDev> sd{sg.sh.dev(nt, NumRec, 0, sg.d_srcv.as<float>(), sg.d_rec.as<float>())};
    TRY(upload(sg.d_shot, sd, st));

    StepSet ps;
    ps.pm = base_params(acc, dt, store_snap, FWI_SNAP_F32, FWI_GRAD_F32, sg.d_fA.as<float>(), sg.d_fB.as<float>());
    ps.pm.items = sg.d_items_m.as<WorkItem>();
    ps.pm.nitems = (int)(adj ? lists.int_adj.size() : lists.int_fwd.size());
    ps.pm.shots = sg.d_shot.as<ShotDev>();
    ps.pm.srcs = sg.d_src.as<SrcEnt>();
    ps.pm.recs = sg.d_recs.as<RecEnt>();
    ps.pm.record = adj ? 0 : 1;
    ps.pb = ps.pm;
    ps.pb.items = sg.d_items_b.as<WorkItem>();
    ps.pb.nitems = (int)(adj ? lists.bnd_adj.size() : lists.bnd_fwd.size());
    ps.pb.nstrip = lists.nstrip;
    ps.kstrip = lists.kstrip;
    // pairs of steps as two-step passes (FP32 snapshots: a pass may store or image)
    const TwoStep tw = two_step_set(ps, adj ? 1 : 0, sg.d_items_f, (int)(adj ? lists.fus_adj : lists.fus_fwd).size(),
                                    lists.ncore, sg.d_items_l, (int)(adj ? lists.lft_adj : lists.lft_fwd).size(),
                                    L().tile_var);
    TRY(run_time_loop(acc, adj ? 1 : 0, nt, store_snap, nt_store, iprop == 1, ps, st, L().aux,
                      lists.fus_fwd.empty() ? nullptr : &tw));

    if (!adj) LK(launch_rec_last(sg.d_rec.as<float>(), nt, NumRec, st));
    // outputs
    if (NumRec > 0)
        CK(cudaMemcpyAsync(Rec_point, sg.d_rec.p, (size_t)nt * NumRec * sizeof(float), cudaMemcpyDeviceToHost, st));
    int rc = FWI_OK;
    if (iprop == 1) {
        // blocks 1..nwritten of Fields; block 0 and unwritten blocks untouched
        const int nw = (int)ev.size();
        if (nw > 0) {
            const size_t fbytes = (size_t)ny * nx * (nw + 1) * sizeof(float);
            TRY(sg.d_stage.ensure(fbytes));
            LK(launch_fields_io(sg.d_stage.as<float>(), sg.sh.snaps.as<float>(), ny, nx, l.pitch, off_dn, nw + 1, 0,
                                st));
            const size_t blk = (size_t)ny * nx;
            CK(cudaMemcpyAsync(Fields + blk, sg.d_stage.as<float>() + blk, blk * nw * sizeof(float),
                               cudaMemcpyDeviceToHost, st));
        }
        if (NumRec > 0) rc = check_nonfinite(sg.d_rec.as<float>(), (size_t)nt * NumRec, sg.d_flag, st, "Rec_point");
    } else if (adj) {
        TRY(sg.d_stage.ensure((size_t)ny * nx * sizeof(float)));
        LK(launch_kernel_io(sg.sh.k.as<float>(), sg.d_stage.as<float>(), ny, nx, l.pitch, off_dn, 0, st));
        CK(cudaMemcpyAsync(kernel, sg.d_stage.p, (size_t)ny * nx * sizeof(float), cudaMemcpyDeviceToHost, st));
        rc = check_nonfinite(sg.d_stage.as<float>(), (size_t)ny * nx, sg.d_flag, st, "kernel");
    } else if (NumRec > 0) {
        rc = check_nonfinite(sg.d_rec.as<float>(), (size_t)nt * NumRec, sg.d_flag, st, "Rec_point");
    }
    CK(cudaStreamSynchronize(st));
    return rc;
}

int fwi_misfit_function(const int* rank, const float* freq, const float* synth, const float* trace, const int* NumRec_,
                        const int* nt_, const float* dt_, float* Misfit, float* AdjSource, double* misfit64) {
    (void)rank;
    (void)freq;
    std::lock_guard<std::recursive_mutex> g(L().mu);
    TRY(ensure_init());
    if (!NumRec_ || !nt_ || !dt_ || !synth || !trace || !Misfit || !AdjSource) return fail(FWI_ERR_ARG, "null argument");
    const int nrec = *NumRec_, nt = *nt_;
    if (nrec < 0 || nt < 1) return fail(FWI_ERR_ARG, "NumRec must be >= 0 and nt >= 1");
    cudaStream_t st = stream();
    const size_t n = (size_t)nrec * nt;
    DBuf ds, dob, da, dtr, doff, dms;
    TRY(ds.alloc(n * 4));
    TRY(dob.alloc(n * 4));
    TRY(da.alloc(n * 4));
    TRY(dtr.alloc(std::max(nrec, 1) * sizeof(double)));
    TRY(doff.alloc(2 * sizeof(int)));
    TRY(dms.alloc(sizeof(double)));
    CK(cudaMemcpyAsync(ds.p, synth, n * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dob.p, trace, n * 4, cudaMemcpyHostToDevice, st));
    const int off[2] = {0, nrec};
    CK(cudaMemcpyAsync(doff.p, off, sizeof off, cudaMemcpyHostToDevice, st));
    LK(launch_misfit(ds.as<float>(), dob.as<float>(), da.as<float>(), dtr.as<double>(), nt, *dt_, doff.as<int>(), nrec,
                     1, dms.as<double>(), st));
    double m = 0.0;
    CK(cudaMemcpyAsync(AdjSource, da.p, n * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&m, dms.p, sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    *Misfit = (float)m;
    if (misfit64) *misfit64 = m;
    return FWI_OK;
}

int fwi_beta_calculous(const float* Grad, const float* OldGrad, const int* nx_, const int* ny_, float* Beta,
                       double* num64, double* den64) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    TRY(ensure_init());
    if (!Grad || !OldGrad || !nx_ || !ny_ || !Beta) return fail(FWI_ERR_ARG, "null argument");
    const size_t n = (size_t)(*nx_) * (*ny_);
    if (*nx_ < 1 || *ny_ < 1) return fail(FWI_ERR_ARG, "nx, ny must be >= 1");
    cudaStream_t st = stream();
    const bool dev = is_device_ptr(Grad) && is_device_ptr(OldGrad);
    DBuf dg, dog, part, out;
    const float *pg = Grad, *po = OldGrad;
    if (!dev) {
        TRY(dg.alloc(n * 4));
        TRY(dog.alloc(n * 4));
        CK(cudaMemcpyAsync(dg.p, Grad, n * 4, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(dog.p, OldGrad, n * 4, cudaMemcpyHostToDevice, st));
        pg = dg.as<float>();
        po = dog.as<float>();
    }
    const int nb = 304;
    TRY(part.alloc(2 * nb * sizeof(double)));
    TRY(out.alloc(2 * sizeof(double)));
    LK(launch_dot(pg, po, n, part.as<double>(), nb, out.as<double>(), st));
    double h[2];
    CK(cudaMemcpyAsync(h, out.p, sizeof h, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    *Beta = (float)(h[0] / h[1]);
    if (num64) *num64 = h[0];
    if (den64) *den64 = h[1];
    return FWI_OK;
}

// Inputs of the NLCG model kernels: device pointers as given, host arrays
// staged through buffers of this call.
namespace {
int nlcg_inputs(const float* a, const float* b, size_t n, DBuf& da, DBuf& db, const float** pa, const float** pb,
                cudaStream_t st) {
    *pa = a;
    *pb = b;
    if (!is_device_ptr(a)) {
        TRY(da.alloc(n * 4));
        CK(cudaMemcpyAsync(da.p, a, n * 4, cudaMemcpyHostToDevice, st));
        *pa = da.as<float>();
    }
    if (!is_device_ptr(b)) {
        TRY(db.alloc(n * 4));
        CK(cudaMemcpyAsync(db.p, b, n * 4, cudaMemcpyHostToDevice, st));
        *pb = db.as<float>();
    }
    return FWI_OK;
}
}  // namespace

int fwi_first_step(const float* Search, const float* var_orig, const int* nx_, const int* ny_, float* nut) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    TRY(ensure_init());
    if (!Search || !var_orig || !nx_ || !ny_ || !nut) return fail(FWI_ERR_ARG, "null argument");
    if (*nx_ < 1 || *ny_ < 1) return fail(FWI_ERR_ARG, "nx, ny must be >= 1");
    const size_t n = (size_t)(*nx_) * (*ny_);
    cudaStream_t st = stream();
    DBuf ds, dv, dm;
    const float *ps = nullptr, *pv = nullptr;
    TRY(nlcg_inputs(Search, var_orig, n, ds, dv, &ps, &pv, st));
    TRY(dm.alloc(sizeof(unsigned)));
    CK(cudaMemsetAsync(dm.p, 0, sizeof(unsigned), st));
    LK(launch_search_max(ps, pv, n, dm.as<unsigned>(), st));
    unsigned bits = 0;
    CK(cudaMemcpyAsync(&bits, dm.p, sizeof bits, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    float mx;
    std::memcpy(&mx, &bits, sizeof mx);
    *nut = (1.f / 100.f) / mx;  // FWI.f90:175 (mx = 0 gives +Inf, as the reference)
    return FWI_OK;
}

int fwi_model_update(const float* Search, const float* var_orig, const float* step, const int* nx_, const int* ny_,
                     float* lambda) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    TRY(ensure_init());
    if (!Search || !var_orig || !step || !nx_ || !ny_ || !lambda) return fail(FWI_ERR_ARG, "null argument");
    if (*nx_ < 1 || *ny_ < 1) return fail(FWI_ERR_ARG, "nx, ny must be >= 1");
    const size_t n = (size_t)(*nx_) * (*ny_);
    cudaStream_t st = stream();
    DBuf ds, dv, dl;
    const float *ps = nullptr, *pv = nullptr;
    TRY(nlcg_inputs(Search, var_orig, n, ds, dv, &ps, &pv, st));
    const bool dev_out = is_device_ptr(lambda);
    float* pl = lambda;
    if (!dev_out) {
        TRY(dl.alloc(n * 4));
        pl = dl.as<float>();
    }
    LK(launch_model_update(ps, pv, *step, n, pl, st));
    if (!dev_out) CK(cudaMemcpyAsync(lambda, pl, n * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return FWI_OK;
}

int fwi_mcs_geometry(float xs, float shot_depth, float streamer_depth, float near_offset, float drec, float dmodel,
                     int num_rec, int* nxSou, int* nySou, int* nxRec, int* nyRec) {
    if (num_rec < 0 || !(dmodel > 0.f)) return fail(FWI_ERR_ARG, "num_rec >= 0 and dmodel > 0 required");
    const float added_space_model = 0.f;  // no parfile key sets it (modules.f90:153)
    const float pos_shot = added_space_model + fabsf(xs);
    if (nxSou) *nxSou = 1 + (int)ceilf(pos_shot / dmodel);
    if (nySou) *nySou = 1 + (int)ceilf(shot_depth / dmodel);
    for (int irec = 1; irec <= num_rec; ++irec) {
        const float pos_rec = (pos_shot - near_offset) - (float)(irec - 1) * drec;
        if (nxRec) nxRec[irec - 1] = 1 + (int)ceilf(pos_rec / dmodel);
        if (nyRec) nyRec[irec - 1] = 1 + (int)ceilf(streamer_depth / dmodel);
    }
    return FWI_OK;
}

int fwi_ricker(float freq, float dt, int nt, float* out) {
    if (nt < 0 || !out || !(freq > 0.f)) return fail(FWI_ERR_ARG, "bad Ricker arguments");
    const float pi = 3.14159265f, f0 = freq, t0 = 1.5f / f0, tmp = 10.f / f0;
    for (int i = 1; i <= nt; ++i) {
        const float t = (float)(i - 1) * dt;
        const float a = (pi * f0) * (t - t0);
        float s = (1.f - 2.f * (a * a)) * expf(-(1.f * (a * a)));
        if (t >= tmp) s = 0.f;
        out[i - 1] = s;
    }
    return FWI_OK;
}

int fwi_time_rules(const float* lambda, int ny, int nx, float dmodel, float tfin, int store_snap, float* dt, int* nt,
                   int* nt_Store) {
    if (!lambda || ny < 1 || nx < 1 || store_snap < 1 || !dt || !nt || !nt_Store) return fail(FWI_ERR_ARG, "bad args");
    float mx = -INFINITY;
    for (size_t i = 0; i < (size_t)ny * nx; ++i) mx = std::max(mx, lambda[i] / 1000.f);
    if (!(mx > 0.f)) return fail(FWI_ERR_ARG, "lambda must be positive");
    *dt = (dmodel / sqrtf(mx)) / 2.f;
    const int n0 = 1 + (int)ceilf(tfin / *dt);
    const float temp = (float)(n0 / store_snap);
    *nt_Store = (int)ceilf(temp);
    *nt = *nt_Store * store_snap;
    return FWI_OK;
}

}  // extern "C"

// ===========================================================================
// batched survey
// ===========================================================================

struct fwi_survey {
    fwi_survey_desc desc{};
    int nt_store = 0;
    std::vector<ShotGeom> geoms;
    std::vector<Layout> lays;
    std::vector<double> gw, mw;
    std::vector<int> tr_off;  // trace offsets per shot (size nshots+1)
    int ntr = 0;
    int wave = 1, band = 64;
    int tile_var = 1, tile_band = TWO_STEP_BAND;  // two-step kernel and rows per two-step tile
    int tile_eband = 0;                           // rows of the bottom edge band (0: a core-height band)
    // single steps chosen by the tuner over the two-step passes (fused: each
    // step one launch), and the timings it compared (ms per two time steps
    // of the first wave)
    bool single_step = false, fused = false;
    // observed data uploaded on the copy stream by the batch call: the misfit
    // (or a graph launch) waits for obs_ready while obs_pending
    cudaEvent_t obs_ready = nullptr;
    bool obs_pending = false;
    float tune_two_ms = -1.f, tune_single_ms = -1.f, tune_fused_ms = -1.f;
    std::vector<float> tune_ms;                   // tuner: [variant][band candidate] ms per pass (-1: not run)
    std::vector<float> tune_ems;                  // tuner: [edge band candidate] ms per pass
    std::vector<std::vector<int>> waves;  // shot indices per wave
    // resident data
    DBuf d_lambda, d_src, d_obs, d_synth, d_adj, d_mis_tr, d_mis_shot, d_tr_off, d_G, d_grad, d_water, d_fA, d_fB;
    // per-slot state
    std::vector<std::unique_ptr<ShotState>> slots;
    // per-wave lists
    struct WaveDev {
        DBuf items_if, items_ia, items_bf, items_ba, src_f, src_a, recs, shots_f, shots_a, stack;
        DBuf items_ff, items_fa, items_lf, items_la;  // two-step tiles; single-step interior items beside them
        int n_if = 0, n_ia = 0, n_bf = 0, n_ba = 0, n_strip = 0, kstrip = 1;
        int n_ff = 0, n_fa = 0, n_lf = 0, n_la = 0, n_core = 0;
        double fus_cells = 0.0;
        cudaGraphExec_t graph[3] = {nullptr, nullptr, nullptr};
        long long graph_kernels[3] = {0, 0, 0};  // kernel nodes per graph
        int direct_runs[3] = {0, 0, 0};          // runs launched directly since the graph was dropped
        // launch form per direction, chosen by measurement: the first run of
        // a time axis is timed as direct launches, the first replay of its
        // graph as a replay (CUDA events around the wave); a graph slower
        // than the direct launches is dropped for good.  A graph that looks
        // faster is kept only after a second direct run (the first one may
        // be the first pass over freshly allocated buffers) confirms it.
        cudaEvent_t tev[2] = {nullptr, nullptr};
        int timing = 0, timing_gi = 0;            // in flight: 1 direct, 2 graph
        float t_direct[3] = {0.f, 0.f, 0.f}, t_graph[3] = {0.f, 0.f, 0.f};
        bool direct_only[3] = {false, false, false};
        bool recheck[3] = {false, false, false}, rechecked[3] = {false, false, false};
        DBuf save_jobs, restore_jobs;  // checkpoint copies: [ckpt][shot][field]
    };
    std::vector<std::unique_ptr<WaveDev>> wdev;
    std::vector<float> h_fA, h_fB;
    bool lambda_set = false;
    // checkpointed recomputation: C forward steps per segment, J segments,
    // `slots` snapshot blocks per shot; per block its segment and slot
    int rc_C = 0, rc_J = 0, rc_slots = 0;
    std::vector<int> ev, blk_seg, blk_slot;
    ~fwi_survey() {
        if (obs_ready) cudaEventDestroy(obs_ready);
        for (auto& w : wdev) {
            for (auto& gexec : w->graph)
                if (gexec) cudaGraphExecDestroy(gexec);
            for (auto& e : w->tev)
                if (e) cudaEventDestroy(e);
        }
    }
};

namespace {

size_t shot_wave_bytes(const Layout& l, int nt_store, int snap_form, int grad_form) {
    const size_t fb = (size_t)l.nyt * l.pitch * 4;
    const size_t esz = snap_form == FWI_SNAP_F32 ? 4 : 2;
    const size_t sb = (size_t)(nt_store + 1) * l.ny * l.pitch * esz + (size_t)(nt_store + 1) * l.ny * (l.ntiles + 2) * 4;
    const size_t kb = (size_t)l.ny * l.pitch * (grad_form == FWI_GRAD_F64 ? 8 : 4);
    return 10 * fb + sb + kb;
}

// Shot packing: shots sorted by window width (widest first, stable) and cut
// into waves of s->wave shots, so that every wave holds shots of similar
// size and the slots (sized by the widest shot that uses them) waste little.
// Slot buffers are allocated here, once.
int survey_prepare_slots(fwi_survey* s) {
    const auto& D = s->desc;
    std::vector<int> order(D.nshots);
    for (int i = 0; i < D.nshots; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return s->geoms[a].nx > s->geoms[b].nx; });
    s->waves.clear();
    for (int i = 0; i < D.nshots; i += s->wave) {
        std::vector<int> w(order.begin() + i, order.begin() + std::min(D.nshots, i + s->wave));
        s->waves.push_back(w);
    }
    // slots persist across re-plans (their buffers only grow)
    if ((int)s->slots.size() > s->wave) s->slots.resize(s->wave);
    while ((int)s->slots.size() < s->wave) s->slots.emplace_back(new ShotState());
    for (int k = 0; k < s->wave; ++k) {
        Layout big = s->lays[s->waves[0][0]];
        size_t best = 0;
        for (size_t wi = 0; wi < s->waves.size(); ++wi) {
            if (k >= (int)s->waves[wi].size()) continue;
            const Layout& l = s->lays[s->waves[wi][k]];
            const size_t b = (size_t)l.nyt * l.pitch;
            if (b >= best) {
                best = b;
                big = l;
            }
        }
        TRY(s->slots[k]->alloc(big, s->rc_C ? s->rc_slots : s->nt_store + 1, D.snap_form, D.grad_form));
        if (s->rc_C) TRY(s->slots[k]->alloc_rc(s->rc_J - 1));
    }
    return FWI_OK;
}

// Work lists and shot descriptors of every wave for the band height s->band.
int survey_prepare_waves(fwi_survey* s) {
    const auto& D = s->desc;
    cudaStream_t st = stream();
    for (auto& w : s->wdev) {
        for (auto& gexec : w->graph)
            if (gexec) {
                cudaGraphExecDestroy(gexec);
                gexec = nullptr;
            }
        for (auto& e : w->tev)
            if (e) {
                cudaEventDestroy(e);
                e = nullptr;
            }
    }
    s->wdev.clear();
    for (size_t wi = 0; wi < s->waves.size(); ++wi) {
        const auto& w = s->waves[wi];
        std::vector<ShotGeom> g;
        std::vector<Layout> l;
        for (int sh : w) {
            g.push_back(s->geoms[sh]);
            l.push_back(s->lays[sh]);
        }
        Lists lists = build_lists(g, l, s->band,
                                  ((D.flags & (FWI_SURVEY_SINGLE_STEP | FWI_SURVEY_FUSED_STEP)) || s->single_step)
                                      ? 0
                                      : s->tile_band,
                                  s->tile_eband);
        std::unique_ptr<fwi_survey::WaveDev> wd(new fwi_survey::WaveDev());
        TRY(upload(wd->items_if, lists.int_fwd, st));
        TRY(upload(wd->items_ia, lists.int_adj, st));
        TRY(upload(wd->items_bf, lists.bnd_fwd, st));
        TRY(upload(wd->items_ba, lists.bnd_adj, st));
        TRY(upload(wd->items_ff, lists.fus_fwd, st));
        TRY(upload(wd->items_fa, lists.fus_adj, st));
        TRY(upload(wd->items_lf, lists.lft_fwd, st));
        TRY(upload(wd->items_la, lists.lft_adj, st));
        wd->n_ff = (int)lists.fus_fwd.size();
        wd->n_fa = (int)lists.fus_adj.size();
        wd->n_lf = (int)lists.lft_fwd.size();
        wd->n_la = (int)lists.lft_adj.size();
        wd->n_core = lists.ncore;
        wd->fus_cells = lists.fus_cells;
        TRY(upload(wd->src_f, lists.src_fwd, st));
        TRY(upload(wd->src_a, lists.src_adj, st));
        TRY(upload(wd->recs, lists.recs, st));
        wd->n_if = (int)lists.int_fwd.size();
        wd->n_ia = (int)lists.int_adj.size();
        wd->n_bf = (int)lists.bnd_fwd.size();
        wd->n_ba = (int)lists.bnd_adj.size();
        wd->n_strip = lists.nstrip;
        wd->kstrip = lists.kstrip;
        s->wdev.push_back(std::move(wd));
    }
    // per-wave shot descriptors (fwd: sources; adj: adjoint source table)
    for (size_t wi = 0; wi < s->waves.size(); ++wi) {
        const auto& w = s->waves[wi];
        std::vector<ShotDev> f, a;
        std::vector<unsigned char> stk(w.size() * stack_shot_size());
        for (size_t k = 0; k < w.size(); ++k) {
            const int sh = w[k];
            ShotState& ss = *s->slots[k];
            const Layout& l = s->lays[sh];
            ShotDev dv = ss.dev(D.nt, (int)s->geoms[sh].nxR.size(), s->geoms[sh].x0, nullptr,
                                s->d_synth.as<float>() + (size_t)s->tr_off[sh] * D.nt);
            dv.snap_stride = (long long)l.ny * l.pitch;
            dv.ny = l.ny; dv.nx = l.nx; dv.nyt = l.nyt; dv.nxt = l.nxt; dv.off = l.off; dv.pitch = l.pitch;
            dv.ntiles = l.ntiles; dv.dn = l.dn; dv.sl = l.sl; dv.sr = l.sr;
            // forward value table: this shot's sources (packed in shot order)
            size_t soff = 0;
            for (int q = 0; q < sh; ++q) soff += s->geoms[q].nxS.size();
            dv.srcv = s->d_src.as<float>() + soff * D.nt;
            f.push_back(dv);
            dv.srcv = s->d_adj.as<float>() + (size_t)s->tr_off[sh] * D.nt;
            if (s->rc_C) {  // the adjoint runs on the second state while the forward is recomputed
                dv.pf[0] = ss.bst[0].as<float>();
                dv.pf[1] = ss.bst[1].as<float>();
                dv.pf[2] = ss.bst[7].as<float>();
                dv.pf[3] = ss.bst[8].as<float>();
                dv.phx = ss.bst[2].as<float>();
                dv.chx = ss.bst[3].as<float>();
                dv.phy = ss.bst[4].as<float>();
                dv.phy2 = ss.bst[5].as<float>();
                dv.chy = ss.bst[6].as<float>();
            }
            a.push_back(dv);
            fill_stack_shot(stk.data() + k * stack_shot_size(), ss.k.as<float>(), ss.k.as<double>(), s->geoms[sh].x0,
                            l.nx, l.off + l.dn, l.pitch, s->gw[sh]);
        }
        auto& wd = *s->wdev[wi];
        TRY(upload(wd.shots_f, f, st));
        TRY(upload(wd.shots_a, a, st));
        TRY(upload(wd.stack, stk, st));
        if (s->rc_C && s->rc_J > 1) {
            const size_t js = copy_job_size(), per = w.size() * 7;
            std::vector<unsigned char> sv(per * (s->rc_J - 1) * js), rv(sv.size());
            for (int c = 0; c < s->rc_J - 1; ++c)
                for (size_t k = 0; k < w.size(); ++k) {
                    ShotState& ss = *s->slots[k];
                    for (int fi = 0; fi < 7; ++fi) {
                        const size_t idx = (size_t)c * per + k * 7 + fi;
                        unsigned char* cp = ss.ckpt.as<unsigned char>() + ((size_t)c * 7 + fi) * ss.field_bytes;
                        fill_copy_job(sv.data() + idx * js, ss.state(fi), cp, ss.field_bytes);
                        fill_copy_job(rv.data() + idx * js, cp, ss.state(fi), ss.field_bytes);
                    }
                }
            TRY(upload(wd.save_jobs, sv, st));
            TRY(upload(wd.restore_jobs, rv, st));
        }
    }
    CK(cudaStreamSynchronize(st));
    return FWI_OK;
}

// ---- autotuner -------------------------------------------------------------
//
// Timed on the first wave, each candidate after a warm-up (the fastest of
// three timings of a few steps):
//   * the two-step tiles, when the survey runs two-step passes: the kernel
//     (k_step2_interior or k_step2s_interior) and the rows per tile
//     (TILE_BANDS), timed as forward two-step passes of the whole wave (the
//     tiles beside the single-step lists, as a gradient runs them);
//   * the band height of the single-step interior items (BANDS), timed as
//     single steps, when single steps carry a share of the run
//     (FWI_SURVEY_SINGLE_STEP, no two-step tiles, or 16-bit snapshots, whose
//     forward snapshot steps are single steps);
//   * single steps against the chosen two-step passes (when no tile choice is
//     forced): a small wave (one 200 x 400 shot) runs faster in single steps,
//     whose launch groups are fewer than the six of a two-step pass.
// A choice forced in the descriptor is not tuned.  Results are cached per
// (device name, rows, order, CPML, wave size, window widths of the first
// wave, time stepping, snapshot form) in memory and in a text file that
// persists across processes: $FWI_TUNE_CACHE, else
// $XDG_CACHE_HOME/fwi_gb300/tuning.txt or $HOME/.cache/fwi_gb300/tuning.txt
// (FWI_TUNE_CACHE set to an empty string: memory only).

int time_wave0_steps(fwi_survey* s, int steps, float* ms, bool single_only = false);

constexpr int TILE_BANDS[] = {16, 32, 48, 64, 96};  // short tiles: more warps for small grids
constexpr int NTB = 5;
// 1-8: small grids, whose time step is the latency of the row marches (the
// strips and the bottom pad follow a band shorter than their own)
constexpr int BANDS[] = {1, 2, 4, 8, 16, 24, 32, 48, 64};
// edge-tile heights (0: the core tiles' bands): the edge tiles run on the
// pass's critical path beside the single-step lists, so shorter edge tiles
// can pay for their extra halo rows
constexpr int EDGE_BANDS[] = {0, 8, 16, 32};
constexpr int NEB = 4;
constexpr int TUNE_PASSES = 24;

std::string tune_cache_path() {
    const char* e = getenv("FWI_TUNE_CACHE");
    if (e) return std::string(e);
    std::string dir;
    if (const char* x = getenv("XDG_CACHE_HOME")) dir = x;
    else if (const char* h = getenv("HOME")) dir = std::string(h) + "/.cache";
    else return std::string();
    return dir + "/fwi_gb300/tuning.txt";
}

std::map<std::string, std::vector<int>>& tune_mem() {
    static std::map<std::string, std::vector<int>> m;
    return m;
}

// band, tile kernel, tile rows of `key` (memory, then the file: last line wins)
bool tune_lookup(const std::string& key, std::vector<int>& out) {
    auto it = tune_mem().find(key);
    if (it != tune_mem().end()) {
        out = it->second;
        return true;
    }
    const std::string path = tune_cache_path();
    if (path.empty()) return false;
    FILE* f = fopen(path.c_str(), "r");
    if (!f) return false;
    char line[1024];
    bool found = false;
    while (fgets(line, sizeof line, f)) {
        char k[900];
        int b = 0, v = 0, r = 0, e = 0, one = 0;
        const int n = sscanf(line, "%899s %d %d %d %d %d", k, &b, &v, &r, &e, &one);
        if (n >= 5 && key == k && b > 0 && (v == 0 || v == 1) && r > 0 && e >= 0 && one >= 0 && one <= 2) {
            out = {b, v, r, e, n == 6 ? one : 0};
            found = true;
        }
    }
    fclose(f);
    if (found) tune_mem()[key] = out;
    return found;
}

void tune_store(const std::string& key, const std::vector<int>& v) {
    tune_mem()[key] = v;
    const std::string path = tune_cache_path();
    if (path.empty()) return;
    // create the directory chain (best effort; a failure only loses the file cache)
    for (size_t p = path.find('/', 1); p != std::string::npos; p = path.find('/', p + 1))
        mkdir(path.substr(0, p).c_str(), 0755);
    if (FILE* f = fopen(path.c_str(), "a")) {
        fprintf(f, "%s %d %d %d %d %d\n", key.c_str(), v[0], v[1], v[2], v[3], v[4]);
        fclose(f);
    }
}

int tune_plan(fwi_survey* s) {
    const auto& D = s->desc;
    if (D.flags & FWI_SURVEY_FUSED_STEP) s->fused = true;
    bool two = (D.flags & (FWI_SURVEY_SINGLE_STEP | FWI_SURVEY_FUSED_STEP)) == 0;
    if (two) {
        two = false;
        for (int sh : s->waves[0]) two = two || two_step_ok(s->lays[sh]);
    }
    if (D.tile_kernel > 0) s->tile_var = D.tile_kernel - 1;
    if (D.tile_rows > 0) s->tile_band = D.tile_rows;
    if (D.tile_edge_rows > 0) s->tile_eband = D.tile_edge_rows;
    s->tune_ems.assign(NEB, -1.f);
    if (D.band_rows > 0) s->band = D.band_rows;
    s->tune_ms.assign(2 * NTB, -1.f);
    const bool do_band = D.band_rows <= 0 && (!two || D.snap_form != FWI_SNAP_F32);
    const bool do_tiles = two && (D.tile_kernel <= 0 || D.tile_rows <= 0 || D.tile_edge_rows <= 0);
    if (do_band || do_tiles) {
        cudaDeviceProp prop;
        CK(cudaGetDeviceProperties(&prop, L().device));
        std::string key = prop.name;
        for (char& c : key)
            if (c == ' ' || c == '|') c = '_';
        key += "|" + std::to_string(D.ny) + "|" + std::to_string(D.acc) + "|" + std::to_string(D.dpml) + "|" +
               std::to_string(s->wave) + "|" + std::to_string(two ? 2 : 1) + "|" + std::to_string(D.snap_form) +
               "|" + std::to_string(D.tile_kernel) + "|" + std::to_string(D.tile_rows) + "|" +
               std::to_string(D.band_rows) + "|" + std::to_string(D.tile_edge_rows) + "|w";
        for (int sh : s->waves[0]) key += "," + std::to_string(s->geoms[sh].nx);
        std::vector<int> hit;
        if (tune_lookup(key, hit)) {
            if (do_band) s->band = hit[0];
            if (two && D.tile_kernel <= 0) s->tile_var = hit[1];
            if (two && D.tile_rows <= 0) s->tile_band = hit[2];
            if (two && D.tile_edge_rows <= 0) s->tile_eband = hit[3];
            if (two && D.tile_kernel <= 0 && D.tile_rows <= 0 && D.tile_edge_rows <= 0) {
                s->single_step = hit[4] != 0;
                s->fused = hit[4] == 2;
                if (s->single_step && D.band_rows <= 0) s->band = hit[0];
            }
        } else {
            if (do_band) {
                // single steps: the two-step lists play no part
                int best = 64;
                float best_ms = 1e30f;
                for (int c : BANDS) {
                    if (c > D.ny && c != BANDS[0]) break;
                    s->band = c;
                    TRY(survey_prepare_waves(s));
                    float ms = 0.f, m = 1e30f;
                    TRY(time_wave0_steps(s, 2, &ms, true));  // warm-up
                    for (int r = 0; r < 3; ++r) {
                        TRY(time_wave0_steps(s, 4, &ms, true));
                        m = std::min(m, ms);
                    }
                    if (m < best_ms) {
                        best_ms = m;
                        best = c;
                    }
                }
                s->band = best;
            }
            // one timing of TUNE_PASSES forward passes: the fastest of three runs
            // after a warm-up (a few passes alone read too fast: the measured
            // order then differs from the order of long runs)
            auto time_passes = [&](float* out) -> int {
                float ms = 0.f, m = 1e30f;
                TRY(time_wave0_steps(s, 8, &ms));
                for (int r = 0; r < 3; ++r) {
                    TRY(time_wave0_steps(s, 2 * TUNE_PASSES, &ms));
                    m = std::min(m, ms);
                }
                *out = m / TUNE_PASSES;
                return FWI_OK;
            };
            if (do_tiles && (D.tile_kernel <= 0 || D.tile_rows <= 0)) {
                // kernel and tile height, with the edge tiles in the core tiles' bands
                const int keep_eb = s->tile_eband;
                if (D.tile_edge_rows <= 0) s->tile_eband = 0;
                float best_ms = 1e30f;
                int bv = s->tile_var, bb = s->tile_band;
                for (int c = 0; c < NTB; ++c) {
                    const int fb = D.tile_rows > 0 ? D.tile_rows : TILE_BANDS[c];
                    if (D.tile_rows > 0 && c > 0) break;
                    s->tile_band = fb;
                    TRY(survey_prepare_waves(s));
                    for (int v = 0; v < 2; ++v) {
                        if (D.tile_kernel > 0 && v != D.tile_kernel - 1) continue;
                        s->tile_var = v;
                        float m = 0.f;
                        TRY(time_passes(&m));
                        s->tune_ms[v * NTB + c] = m;
                        if (m < best_ms) {
                            best_ms = m;
                            bv = v;
                            bb = fb;
                        }
                    }
                }
                s->tile_var = bv;
                s->tile_band = bb;
                s->tile_eband = keep_eb;
            }
            if (do_tiles && D.tile_edge_rows <= 0) {
                // then the edge tiles' height for that kernel and tile height
                float best_ms = 1e30f;
                int be = 0;
                for (int c = 0; c < NEB; ++c) {
                    if (EDGE_BANDS[c] >= s->tile_band) continue;
                    s->tile_eband = EDGE_BANDS[c];
                    TRY(survey_prepare_waves(s));
                    float m = 0.f;
                    TRY(time_passes(&m));
                    s->tune_ems[c] = m;
                    if (m < best_ms) {
                        best_ms = m;
                        be = EDGE_BANDS[c];
                    }
                }
                s->tile_eband = be;
            }
            if (two && D.tile_kernel <= 0 && D.tile_rows <= 0 && D.tile_edge_rows <= 0) {
                // the chosen two-step passes against single steps (their band
                // height tuned too, unless forced), each per two time steps
                float m2 = 0.f;
                TRY(survey_prepare_waves(s));
                TRY(time_passes(&m2));
                const int keep_band = s->band;
                float m1 = 1e30f;
                int b1 = keep_band;
                s->single_step = true;
                for (int c : BANDS) {
                    const int bb = D.band_rows > 0 ? D.band_rows : c;
                    if (D.band_rows > 0 && c != BANDS[0]) break;
                    if (bb > D.ny && c != BANDS[0]) break;
                    s->band = bb;
                    TRY(survey_prepare_waves(s));
                    float ms = 0.f, m = 1e30f;
                    TRY(time_wave0_steps(s, 8, &ms, true));
                    for (int r = 0; r < 3; ++r) {
                        TRY(time_wave0_steps(s, 2 * TUNE_PASSES, &ms, true));
                        m = std::min(m, ms);
                    }
                    m /= TUNE_PASSES;
                    if (m < m1) {
                        m1 = m;
                        b1 = bb;
                    }
                }
                // single steps in one launch each (the fused kernel), at that band
                s->band = b1;
                s->fused = true;
                TRY(survey_prepare_waves(s));
                float mf = 1e30f, ms = 0.f;
                TRY(time_wave0_steps(s, 8, &ms, true));
                for (int r = 0; r < 3; ++r) {
                    TRY(time_wave0_steps(s, 2 * TUNE_PASSES, &ms, true));
                    mf = std::min(mf, ms);
                }
                mf /= TUNE_PASSES;
                s->tune_two_ms = m2;
                s->tune_single_ms = m1;
                s->tune_fused_ms = mf;
                // single steps only where they are clearly faster (2 %)
                s->single_step = std::min(m1, mf) < 0.98f * m2;
                s->fused = s->single_step && mf < m1;
                s->band = s->single_step ? b1 : keep_band;
            }
            tune_store(key, {s->band, s->tile_var, s->tile_band, s->tile_eband,
                             s->single_step ? (s->fused ? 2 : 1) : 0});
        }
        if (two) {
            L().tile_var = s->tile_var;
            L().tile_band = s->single_step ? 0 : s->tile_band;
            L().tile_eband = s->tile_eband;
        }
    }
    return survey_prepare_waves(s);
}

// ---- checkpointed recomputation -------------------------------------------
//
// Segment j holds forward steps k in [C*j+1, C*(j+1)].  The forward run keeps
// the full state after steps C, 2C, ... (checkpoints) and the snapshots of
// the last segment only; the adjoint, which consumes snapshot blocks from the
// last to the first, re-runs the forward of a segment from its checkpoint
// into the small snapshot ring whenever it needs a block of another segment.
// The arithmetic of every step is unchanged, so the gradient is identical to
// the one computed with all snapshots stored.

int rc_plan(fwi_survey* s, int C) {
    const auto& D = s->desc;
    s->rc_C = C;
    s->ev = snapshot_steps(D.nt, D.store_snap);
    s->rc_J = (D.nt - 1) / C + 1;
    const int nb = (int)s->ev.size();
    s->blk_seg.assign(nb + 1, 0);
    s->blk_slot.assign(nb + 1, 0);
    std::vector<int> first(s->rc_J, -1);
    for (int b = 1; b <= nb; ++b) {
        const int j = (s->ev[b - 1] - 1) / C;
        s->blk_seg[b] = j;
        if (first[j] < 0) first[j] = b;
        s->blk_slot[b] = b - first[j] + 1;  // slot 0 is block 0 (zeros) in segment 0
    }
    int mx = 0;
    for (int b = 1; b <= nb; ++b) mx = std::max(mx, s->blk_slot[b]);
    s->rc_slots = mx + 1;
    return FWI_OK;
}

int zero_slot0(fwi_survey* s, size_t wi, cudaStream_t st) {
    const auto& D = s->desc;
    for (size_t k = 0; k < s->waves[wi].size(); ++k) {
        ShotState& ss = *s->slots[k];
        const Layout& l = s->lays[s->waves[wi][k]];
        const size_t esz = D.snap_form == FWI_SNAP_F32 ? 4 : 2;
        CK(cudaMemsetAsync(ss.snaps.p, 0, (size_t)l.ny * l.pitch * esz, st));
        CK(cudaMemsetAsync(ss.sscale.p, 0, (size_t)l.ny * (l.ntiles + 2) * sizeof(float), st));
    }
    return FWI_OK;
}

// Forward steps k0..k1 on state A; snapshots of blocks whose segment is
// `keep_seg` go to their ring slots (keep_seg < 0: none).  With save_ckpt the
// state is saved after every checkpoint step (a multiple of C); the steps in
// between run as two-step passes and single steps (run_range), so the state
// is in pair 0 at every save.
int rc_steps(fwi_survey* s, int k0, int k1, int keep_seg, bool save_ckpt, size_t wi, StepSet ps, const TwoStep* tw,
             cudaStream_t st, cudaStream_t st2) {
    const auto& D = s->desc;
    auto& wd = *s->wdev[wi];
    const int per = (int)s->waves[wi].size() * 7;
    std::vector<int> sn(k1 + 2, -1);
    for (size_t i = 0; i < s->ev.size(); ++i) {
        const int e = s->ev[i], b = (int)i + 1;
        if (e >= k0 && e <= k1 && s->blk_seg[b] == keep_seg) sn[e] = s->blk_slot[b];
    }
    auto sn_of = [&](int k) { return sn[k]; };
    int k = k0;
    while (k <= k1) {
        int e = k1;
        bool save = false;
        if (save_ckpt) {
            const int c = (k + s->rc_C - 1) / s->rc_C * s->rc_C;  // first multiple of C at or after k
            if (c <= k1 && c / s->rc_C <= s->rc_J - 1) {
                e = c;
                save = true;
            }
        }
        TRY(run_range(D.acc, 0, k, e, sn_of, ps, tw, st, st2));
        if (save) {
            const int c = e / s->rc_C - 1;
            LK(launch_copy_jobs(wd.save_jobs.as<unsigned char>() + (size_t)c * per * copy_job_size(), per, st));
        }
        k = e + 1;
    }
    return FWI_OK;
}

int rc_forward(fwi_survey* s, size_t wi, int step, StepSet ps, const TwoStep* tw, cudaStream_t st,
               cudaStream_t st2) {
    // keep the last segment's snapshots (the adjoint needs them first)
    if (step == 1 && s->rc_J == 1) TRY(zero_slot0(s, wi, st));
    return rc_steps(s, 2, s->desc.nt, step == 1 ? s->rc_J - 1 : -1, step == 1, wi, ps, tw, st, st2);
}

int rc_recompute(fwi_survey* s, size_t wi, int j, StepSet psf, const TwoStep* twf, cudaStream_t st,
                 cudaStream_t st2) {
    auto& wd = *s->wdev[wi];
    const int per = (int)s->waves[wi].size() * 7;
    if (j == 0) {
        for (size_t k = 0; k < s->waves[wi].size(); ++k) {
            ShotState& ss = *s->slots[k];
            for (int fi = 0; fi < 7; ++fi) CK(cudaMemsetAsync(ss.state(fi), 0, ss.field_bytes, st));
        }
        TRY(zero_slot0(s, wi, st));
    } else {
        LK(launch_copy_jobs(wd.restore_jobs.as<unsigned char>() + (size_t)(j - 1) * per * copy_job_size(), per, st));
    }
    const int k0 = std::max(2, s->rc_C * j + 1), k1 = std::min(s->desc.nt, s->rc_C * (j + 1));
    return rc_steps(s, k0, k1, j, false, wi, psf, twf, st, st2);
}

int rc_adjoint(fwi_survey* s, size_t wi, StepSet ps, cudaStream_t st, cudaStream_t st2) {
    const auto& D = s->desc;
    auto& wd = *s->wdev[wi];
    StepSet psf;  // forward recompute: state A, no receivers
    psf.pm = ps.pm;
    psf.pm.items = wd.items_if.as<WorkItem>();
    psf.pm.nitems = wd.n_if;
    psf.pm.shots = wd.shots_f.as<ShotDev>();
    psf.pm.srcs = wd.src_f.as<SrcEnt>();
    psf.pm.record = 0;
    psf.pb = psf.pm;
    psf.pb.items = wd.items_bf.as<WorkItem>();
    psf.pb.nitems = wd.n_bf;
    psf.pb.nstrip = wd.n_strip;
    psf.kstrip = wd.kstrip;
    psf.fused = s->fused;
    ps.pm.items = wd.items_ia.as<WorkItem>();
    ps.pm.nitems = wd.n_ia;
    ps.pm.shots = wd.shots_a.as<ShotDev>();
    ps.pm.srcs = wd.src_a.as<SrcEnt>();
    ps.pm.record = 0;
    ps.pb = ps.pm;
    ps.pb.items = wd.items_ba.as<WorkItem>();
    ps.pb.nitems = wd.n_ba;
    ps.pb.nstrip = wd.n_strip;
    ps.kstrip = wd.kstrip;
    ps.fused = s->fused;
    const TwoStep twf = two_step_set(psf, 0, wd.items_ff, wd.n_ff, wd.n_core, wd.items_lf, wd.n_lf, s->tile_var);
    const TwoStep twa = two_step_set(ps, 1, wd.items_fa, wd.n_fa, wd.n_core, wd.items_la, wd.n_la, s->tile_var);
    const TwoStep* pf = wd.n_ff ? &twf : nullptr;
    const TwoStep* pa = wd.n_fa ? &twa : nullptr;
    // imaging steps: the block each uses (solver_acoustic_SS.f90:460) and its
    // slot in the snapshot ring; a block of another segment than the ring
    // holds is recomputed first, so the adjoint runs in ranges between those
    std::vector<int> sn(D.nt + 2, -1), need(D.nt + 2, -1);
    int snap = s->nt_store;
    for (int e : s->ev) {
        --snap;
        sn[e] = snap == 0 ? 0 : s->blk_slot[snap];
        need[e] = snap == 0 ? 0 : s->blk_seg[snap];
    }
    auto sn_of = [&](int k) { return sn[k]; };
    int cur = s->rc_J - 1;
    int k = 2;
    for (int e : s->ev) {
        if (need[e] == cur) continue;
        TRY(run_range(D.acc, 1, k, e - 1, sn_of, ps, pa, st, st2));
        TRY(rc_recompute(s, wi, need[e], psf, pf, st, st2));
        cur = need[e];
        k = e;
    }
    return run_range(D.acc, 1, k, D.nt, sn_of, ps, pa, st, st2);
}

// Issue one wave's work: forward (+ misfit) and, for step 1, adjoint + stack.
int issue_wave(fwi_survey* s, size_t wi, int step, cudaStream_t st, cudaStream_t st2) {
    const auto& D = s->desc;
    const auto& w = s->waves[wi];
    auto& wd = *s->wdev[wi];
    for (size_t k = 0; k < w.size(); ++k) {
        const int sh = w[k];
        ShotState& ss = *s->slots[k];
        const Layout& l = s->lays[sh];
        // the slot may be larger than this shot: zero the whole allocation
        CK(cudaMemsetAsync(ss.pa.p, 0, ss.pa.n, st));
        CK(cudaMemsetAsync(ss.pb.p, 0, ss.pb.n, st));
        CK(cudaMemsetAsync(ss.pc.p, 0, ss.pc.n, st));
        CK(cudaMemsetAsync(ss.pd.p, 0, ss.pd.n, st));
        CK(cudaMemsetAsync(ss.phx.p, 0, ss.phx.n, st));
        CK(cudaMemsetAsync(ss.chx.p, 0, ss.chx.n, st));
        CK(cudaMemsetAsync(ss.phy.p, 0, ss.phy.n, st));
        CK(cudaMemsetAsync(ss.phy2.p, 0, ss.phy2.n, st));
        CK(cudaMemsetAsync(ss.chy.p, 0, ss.chy.n, st));
        CK(cudaMemsetAsync(ss.c2.p, 0, ss.c2.n, st));
        // snapshot block 0 is never written by the forward but is the last
        // one the adjoint pairs with: zero, as Fields = 0 before the forward
        // (calculate_misfit_gradient.f90:231)
        if (step == 1 && !s->rc_C) {
            const size_t esz = D.snap_form == FWI_SNAP_F32 ? 4 : 2;
            CK(cudaMemsetAsync(ss.snaps.p, 0, (size_t)l.ny * l.pitch * esz, st));
            CK(cudaMemsetAsync(ss.sscale.p, 0, (size_t)l.ny * (l.ntiles + 2) * sizeof(float), st));
        }
        LK(launch_build_c2(ss.c2.as<float>(), l.nyt, l.pitch, l.off, l.dn, l.ny, l.nx, s->d_lambda.as<float>(), D.ny,
                           s->geoms[sh].x0, 1, D.dt * D.dt, D.d * D.d, st));
        float* rec = s->d_synth.as<float>() + (size_t)s->tr_off[sh] * D.nt;
        CK(cudaMemsetAsync(rec, 0, (size_t)(int)s->geoms[sh].nxR.size() * D.nt * sizeof(float), st));
    }
    StepSet ps;
    ps.pm = base_params(D.acc, D.dt, D.store_snap, D.snap_form, D.grad_form, s->d_fA.as<float>(), s->d_fB.as<float>());
    ps.pm.items = wd.items_if.as<WorkItem>();
    ps.pm.nitems = wd.n_if;
    ps.pm.shots = wd.shots_f.as<ShotDev>();
    ps.pm.srcs = wd.src_f.as<SrcEnt>();
    ps.pm.recs = wd.recs.as<RecEnt>();
    ps.pm.record = 1;
    ps.pb = ps.pm;
    ps.pb.items = wd.items_bf.as<WorkItem>();
    ps.pb.nitems = wd.n_bf;
    ps.pb.nstrip = wd.n_strip;
    ps.kstrip = wd.kstrip;
    ps.fused = s->fused;
    {
        const TwoStep tw = two_step_set(ps, 0, wd.items_ff, wd.n_ff, wd.n_core, wd.items_lf, wd.n_lf, s->tile_var);
        const TwoStep* ptw = wd.n_ff ? &tw : nullptr;
        if (s->rc_C) TRY(rc_forward(s, wi, step, ps, ptw, st, st2));
        else TRY(run_time_loop(D.acc, 0, D.nt, D.store_snap, s->nt_store, step == 1, ps, st, st2, ptw));
    }
    for (size_t k = 0; k < w.size(); ++k) {
        const int sh = w[k];
        LK(launch_rec_last(s->d_synth.as<float>() + (size_t)s->tr_off[sh] * D.nt, D.nt, (int)s->geoms[sh].nxR.size(), st));
    }
    // misfit + adjoint source for this wave's traces (one launch per shot:
    // the shots of a wave need not be consecutive); the observed data may
    // still be on their way (the batch call uploads them beside the forward
    // pass and records obs_ready before it launches a wave); a captured wave
    // waits for that event inside its graph
    {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        CK(cudaStreamIsCapturing(st, &cs));
        if (cs == cudaStreamCaptureStatusActive) CK(cudaStreamWaitEvent(st, s->obs_ready, cudaEventWaitExternal));
        else if (s->obs_pending) CK(cudaStreamWaitEvent(st, s->obs_ready, 0));
    }
    for (int sh : w) {
        const int t0 = s->tr_off[sh], t1 = s->tr_off[sh + 1];
        if (t1 == t0) continue;
        LK(launch_misfit(s->d_synth.as<float>() + (size_t)t0 * D.nt, s->d_obs.as<float>() + (size_t)t0 * D.nt,
                         s->d_adj.as<float>() + (size_t)t0 * D.nt, s->d_mis_tr.as<double>() + t0, D.nt, D.dt,
                         s->d_tr_off.as<int>(), t1 - t0, 0, nullptr, st));
    }
    if (step != 1) return FWI_OK;
    for (size_t k = 0; k < w.size(); ++k) {
        ShotState& ss = *s->slots[k];
        for (int fi = 0; fi < 7; ++fi) {
            void* f = s->rc_C ? ss.bst[fi].p : ss.state(fi);
            CK(cudaMemsetAsync(f, 0, ss.field_bytes, st));
        }
        if (s->rc_C) {  // the adjoint's second wavefield pair (its top pad must read zero)
            CK(cudaMemsetAsync(ss.bst[7].p, 0, ss.field_bytes, st));
            CK(cudaMemsetAsync(ss.bst[8].p, 0, ss.field_bytes, st));
        }
        CK(cudaMemsetAsync(ss.k.p, 0, ss.k.n, st));
    }
    if (s->rc_C) {
        TRY(rc_adjoint(s, wi, ps, st, st2));
        LK(launch_stack(s->d_G.as<double>(), D.ny, D.nx_model, wd.stack.p, (int)w.size(), D.grad_form, st));
        return FWI_OK;
    }
    ps.pm.items = wd.items_ia.as<WorkItem>();
    ps.pm.nitems = wd.n_ia;
    ps.pm.shots = wd.shots_a.as<ShotDev>();
    ps.pm.srcs = wd.src_a.as<SrcEnt>();
    ps.pm.record = 0;
    ps.pb = ps.pm;
    ps.pb.items = wd.items_ba.as<WorkItem>();
    ps.pb.nitems = wd.n_ba;
    ps.pb.nstrip = wd.n_strip;
    ps.kstrip = wd.kstrip;
    ps.fused = s->fused;
    TwoStep tw = two_step_set(ps, 1, wd.items_fa, wd.n_fa, wd.n_core, wd.items_la, wd.n_la, s->tile_var);
    TRY(run_time_loop(D.acc, 1, D.nt, D.store_snap, s->nt_store, true, ps, st, st2, wd.n_fa ? &tw : nullptr));
    LK(launch_stack(s->d_G.as<double>(), D.ny, D.nx_model, wd.stack.p, (int)w.size(), D.grad_form, st));
    return FWI_OK;
}

}  // namespace

// Time-axis plan of a survey: the wave size from the HBM budget (the memory
// the survey's slots already hold counts as available), checkpointed
// recomputation when waves would get too small, the slots (reused; their
// buffers only grow), the band height and the work lists of every wave.
int survey_plan(fwi_survey* s, bool tune) {
    const auto& D = s->desc;
    s->rc_C = 0;
    size_t held = 0;
    for (auto& sl : s->slots) held += sl->bytes();
    // wave size from the HBM budget
    size_t per = 0;
    for (auto& l : s->lays) per = std::max(per, shot_wave_bytes(l, s->nt_store, D.snap_form, D.grad_form));
    size_t freeb = 0, totb = 0;
    CK(cudaMemGetInfo(&freeb, &totb));
    size_t budget = (size_t)(0.92 * (double)(freeb + held));
    if (s->desc.hbm_budget) {
        size_t used_resident = s->d_obs.n + s->d_synth.n + s->d_adj.n + s->d_src.n + s->d_G.n + s->d_lambda.n;
        if (s->desc.hbm_budget <= used_resident) return fail(FWI_ERR_NOMEM, "HBM budget smaller than the resident data");
        budget = std::min(budget, s->desc.hbm_budget - used_resident);
    }
    int wave = (int)std::min<size_t>((size_t)D.nshots, budget / std::max<size_t>(per, 1));
    // Checkpointed recomputation keeps a forward-state checkpoint every C steps
    // and a ring of C/store_snap snapshots instead of all of them, for one more
    // forward pass.  It is used when asked for, or when the budget would leave
    // waves so small (< 8 shots) that the extra pass is cheaper than the lost
    // batching.
    {
        size_t fb = 0, bb = 0, kb = 0;
        for (auto& l : s->lays) {
            fb = std::max(fb, (size_t)l.nyt * l.pitch * 4);
            bb = std::max(bb, (size_t)l.ny * l.pitch * (D.snap_form == FWI_SNAP_F32 ? 4 : 2) + (size_t)l.ny * (l.ntiles + 2) * 4);
            kb = std::max(kb, (size_t)l.ny * l.pitch * (D.grad_form == FWI_GRAD_F64 ? 8 : 4));
        }
        const int ss = D.store_snap;
        int C = (int)std::lround(std::sqrt(7.0 * fb * D.nt * ss / (double)std::max<size_t>(bb, 1)));
        C = std::max(ss, std::min(D.nt, (C + ss - 1) / ss * ss));
        const int J = (D.nt - 1) / C + 1;
        const size_t per_rc = 19 * fb + (size_t)(J - 1) * 7 * fb + (size_t)(C / ss + 2) * bb + kb;
        const int wave_rc = (int)std::min<size_t>((size_t)D.nshots, budget / std::max<size_t>(per_rc, 1));
        const bool force = (D.flags & FWI_SURVEY_RECOMPUTE) != 0;
        if (force || (wave < std::min(D.nshots, 8) && wave_rc > wave)) {
            if (wave_rc < 1)
                return fail(FWI_ERR_NOMEM, "one shot's checkpoints and snapshot ring (" + std::to_string(per_rc) +
                                               " bytes) exceed the device budget");
            TRY(rc_plan(s, C));
            wave = wave_rc;
        }
    }
    if (wave < 1)
        return fail(FWI_ERR_NOMEM, "one shot's wavefields and snapshots (" + std::to_string(per) +
                                       " bytes) exceed the device budget");
    if (D.wave_shots > 0) wave = std::min(wave, D.wave_shots);
    // balance the waves: same number of shots in each
    const int nw = (D.nshots + wave - 1) / wave;
    wave = (D.nshots + nw - 1) / nw;
    s->wave = wave;
    TRY(survey_prepare_slots(s));
    if (tune) return tune_plan(s);
    if (D.band_rows > 0) s->band = D.band_rows;
    return survey_prepare_waves(s);
}

extern "C" {

int fwi_survey_create(const fwi_survey_desc* desc, fwi_survey** out) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    TRY(ensure_init());
    if (!desc || !out) return fail(FWI_ERR_ARG, "null argument");
    const fwi_survey_desc& D = *desc;
    TRY(validate_common(D.ny, D.nx_model, D.acc, D.dpml, D.nt, D.store_snap));
    if (D.nshots < 1 || !D.shots) return fail(FWI_ERR_ARG, "nshots must be >= 1");
    if (!(D.d > 0.f) || !(D.dt > 0.f)) return fail(FWI_ERR_ARG, "d and dt must be positive");
    if (D.numtasks < 1) return fail(FWI_ERR_ARG, "numtasks must be >= 1");
    if (D.snap_form < 0 || D.snap_form > 2 || D.grad_form < 0 || D.grad_form > 1)
        return fail(FWI_ERR_ARG, "bad snap_form / grad_form");
    std::unique_ptr<fwi_survey> s(new fwi_survey());
    s->desc = D;
    CK(cudaEventCreateWithFlags(&s->obs_ready, cudaEventDisableTiming));
    s->nt_store = D.nt / D.store_snap;
    if ((int)snapshot_steps(D.nt, D.store_snap).size() > s->nt_store)
        return fail(FWI_ERR_ARG, "nt/store_snap snapshots exceed nt_Store");
    s->tr_off.assign(D.nshots + 1, 0);
    int nsou_tot = 0;
    for (int i = 0; i < D.nshots; ++i) {
        const fwi_shot& sh = D.shots[i];
        if (sh.nx < 1 || sh.x0 < 0 || sh.x0 + sh.nx > D.nx_model)
            return fail(FWI_ERR_ARG, "shot " + std::to_string(i) + ": window outside the model");
        if (sh.num_sou < 0 || sh.num_rec < 0) return fail(FWI_ERR_ARG, "negative source/receiver count");
        if ((sh.num_sou && (!sh.nxSou || !sh.nySou)) || (sh.num_rec && (!sh.nxRec || !sh.nyRec)))
            return fail(FWI_ERR_ARG, "shot " + std::to_string(i) + ": null geometry arrays");
        ShotGeom geo;
        geo.x0 = sh.x0;
        geo.nx = sh.nx;
        geo.nxS.assign(sh.nxSou, sh.nxSou + sh.num_sou);
        geo.nyS.assign(sh.nySou, sh.nySou + sh.num_sou);
        geo.nxR.assign(sh.nxRec, sh.nxRec + sh.num_rec);
        geo.nyR.assign(sh.nyRec, sh.nyRec + sh.num_rec);
        const Layout l = make_layout(D.ny, sh.nx, D.acc, D.dpml);
        TRY(validate_geometry(geo, l, i + 1));
        s->geoms.push_back(geo);
        s->lays.push_back(l);
        s->gw.push_back(sh.grad_weight);
        s->mw.push_back(sh.misfit_weight);
        s->tr_off[i + 1] = s->tr_off[i] + sh.num_rec;
        nsou_tot += sh.num_sou;
    }
    s->ntr = s->tr_off[D.nshots];
    cudaStream_t st = stream();
    const size_t nt = D.nt;
    // resident data
    TRY(s->d_lambda.alloc((size_t)D.ny * D.nx_model * 4));
    TRY(s->d_src.alloc(std::max<size_t>(nt * nsou_tot * 4, 16)));
    TRY(s->d_obs.alloc(std::max<size_t>(nt * s->ntr * 4, 16)));
    TRY(s->d_synth.alloc(std::max<size_t>(nt * s->ntr * 4, 16)));
    TRY(s->d_adj.alloc(std::max<size_t>(nt * s->ntr * 4, 16)));
    TRY(s->d_mis_tr.alloc(std::max<size_t>(s->ntr * 8, 16)));
    TRY(s->d_mis_shot.alloc(D.nshots * 8));
    TRY(upload(s->d_tr_off, s->tr_off, st));
    TRY(s->d_G.alloc((size_t)D.ny * D.nx_model * 8));
    TRY(s->d_grad.alloc((size_t)D.ny * D.nx_model * 4));
    if (D.water_rows) {
        std::vector<int> w(D.water_rows, D.water_rows + D.nx_model);
        TRY(upload(s->d_water, w, st));
    }
    pml_factors(D.acc, D.dpml, D.dt, D.d, s->h_fA, s->h_fB);
    TRY(upload(s->d_fA, s->h_fA, st));
    TRY(upload(s->d_fB, s->h_fB, st));
    {
        size_t so = 0, to = 0;
        for (int i = 0; i < D.nshots; ++i) {
            const fwi_shot& sh = D.shots[i];
            if (sh.num_sou && sh.src)
                CK(cudaMemcpyAsync(s->d_src.as<float>() + so, sh.src, nt * sh.num_sou * 4, cudaMemcpyHostToDevice, st));
            else if (sh.num_sou)
                CK(cudaMemsetAsync(s->d_src.as<float>() + so, 0, nt * sh.num_sou * 4, st));
            if (sh.num_rec && sh.obs)
                CK(cudaMemcpyAsync(s->d_obs.as<float>() + to, sh.obs, nt * sh.num_rec * 4, cudaMemcpyHostToDevice, st));
            else if (sh.num_rec)
                CK(cudaMemsetAsync(s->d_obs.as<float>() + to, 0, nt * sh.num_rec * 4, st));
            so += nt * sh.num_sou;
            to += nt * sh.num_rec;
        }
    }
    CK(cudaStreamSynchronize(st));
    s->desc.shots = nullptr;  // host pointers are not kept
    TRY(survey_plan(s.get(), true));
    *out = s.release();
    return FWI_OK;
}

int fwi_survey_set_time(fwi_survey* s, float dt, int nt, const float* src, const float* obs) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    if (!s) return fail(FWI_ERR_STATE, "null survey");
    auto& D = s->desc;
    TRY(validate_common(D.ny, D.nx_model, D.acc, D.dpml, nt, D.store_snap));
    if (!(dt > 0.f)) return fail(FWI_ERR_ARG, "dt must be positive");
    if ((int)snapshot_steps(nt, D.store_snap).size() > nt / D.store_snap)
        return fail(FWI_ERR_ARG, "nt/store_snap snapshots exceed nt_Store");
    cudaStream_t st = stream();
    CK(cudaStreamSynchronize(st));
    const bool nt_changed = nt != D.nt;
    size_t nsou_tot = 0;
    for (auto& gm : s->geoms) nsou_tot += gm.nxS.size();
    D.nt = nt;
    D.dt = dt;
    s->nt_store = nt / D.store_snap;
    const size_t nsrc = (size_t)nt * nsou_tot, ntrc = (size_t)nt * s->ntr;
    TRY(s->d_src.ensure(std::max<size_t>(nsrc * 4, 16)));
    TRY(s->d_obs.ensure(std::max<size_t>(ntrc * 4, 16)));
    TRY(s->d_synth.ensure(std::max<size_t>(ntrc * 4, 16)));
    TRY(s->d_adj.ensure(std::max<size_t>(ntrc * 4, 16)));
    // CPML factors depend on dt (solver_PML_coeffs.f90)
    pml_factors(D.acc, D.dpml, D.dt, D.d, s->h_fA, s->h_fB);
    TRY(upload(s->d_fA, s->h_fA, st));
    TRY(upload(s->d_fB, s->h_fB, st));
    auto put = [&](DBuf& dst, const float* p, size_t n) -> int {
        if (!n) return FWI_OK;
        if (p) CK(cudaMemcpyAsync(dst.p, p, n * 4, is_device_ptr(p) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
        else CK(cudaMemsetAsync(dst.p, 0, n * 4, st));
        return FWI_OK;
    };
    TRY(put(s->d_src, src, nsrc));
    TRY(put(s->d_obs, obs, ntrc));
    if (nt_changed) {
        TRY(survey_plan(s, false));
    } else {
        // dt is baked into the captured graphs (c2, the snapshot scaling)
        for (auto& w : s->wdev) {
            for (auto& gexec : w->graph)
                if (gexec) {
                    cudaGraphExecDestroy(gexec);
                    gexec = nullptr;
                }
            for (int& n : w->direct_runs) n = 0;
            for (int i = 0; i < 3; ++i) {
                w->t_direct[i] = w->t_graph[i] = 0.f;
                w->direct_only[i] = w->recheck[i] = w->rechecked[i] = false;
            }
            w->timing = 0;
        }
    }
    CK(cudaStreamSynchronize(st));
    return FWI_OK;
}

int fwi_survey_destroy(fwi_survey* s) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    if (!s) return FWI_OK;
    cudaStreamSynchronize(stream());
    delete s;
    return FWI_OK;
}

int fwi_survey_set_lambda(fwi_survey* s, const float* lambda) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    if (!s || !lambda) return fail(FWI_ERR_STATE, "null survey or lambda");
    const size_t n = (size_t)s->desc.ny * s->desc.nx_model * 4;
    CK(cudaMemcpyAsync(s->d_lambda.p, lambda, n, is_device_ptr(lambda) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                       stream()));
    s->lambda_set = true;
    return FWI_OK;
}

int fwi_survey_set_observed(fwi_survey* s, const float* obs) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    if (!s || !obs) return fail(FWI_ERR_STATE, "null survey or data");
    const size_t n = (size_t)s->ntr * s->desc.nt * 4;
    if (n) CK(cudaMemcpyAsync(s->d_obs.p, obs, n, is_device_ptr(obs) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                              stream()));
    return FWI_OK;
}

int fwi_survey_set_sources(fwi_survey* s, const float* src) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    if (!s || !src) return fail(FWI_ERR_STATE, "null survey or sources");
    size_t nsou = 0;
    for (auto& gg : s->geoms) nsou += gg.nxS.size();
    const size_t n = nsou * s->desc.nt * 4;
    if (n) CK(cudaMemcpyAsync(s->d_src.p, src, n, is_device_ptr(src) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                              stream()));
    return FWI_OK;
}

int fwi_survey_run(fwi_survey* s, int step, double* misfit, float* grad) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    if (!s) return fail(FWI_ERR_STATE, "null survey");
    if (!s->lambda_set) return fail(FWI_ERR_STATE, "fwi_survey_set_lambda has not been called");
    if (step != 1 && step != 2) return fail(FWI_ERR_ARG, "step must be 1 or 2");
    const auto& D = s->desc;
    cudaStream_t st = stream();
    CK(cudaMemsetAsync(s->d_G.p, 0, s->d_G.n, st));
    const int gi = step == 1 ? 0 : 1;
    for (size_t wi = 0; wi < s->waves.size(); ++wi) {
        auto& wd = *s->wdev[wi];
        // the first run of a time axis launches directly: capturing and
        // instantiating a long time loop costs seconds, which a time axis run
        // once (a line-search trial) would not win back; the second run
        // captures the graph, later runs replay it
        const bool no_graph = (D.flags & FWI_SURVEY_NO_GRAPH) != 0;
        if (!wd.tev[0] && !no_graph) {
            CK(cudaEventCreate(&wd.tev[0]));
            CK(cudaEventCreate(&wd.tev[1]));
        }
        const bool graph_only = (D.flags & FWI_SURVEY_GRAPH) != 0;
        if (no_graph ||
            (!graph_only && (wd.direct_only[gi] || wd.recheck[gi] || (!wd.graph[gi] && wd.direct_runs[gi] == 0)))) {
            const bool timed = !no_graph && (wd.t_direct[gi] == 0.f || wd.recheck[gi]);
            if (timed) CK(cudaEventRecord(wd.tev[0], st));
            TRY(issue_wave(s, wi, step, st, L().aux));
            if (timed) {
                CK(cudaEventRecord(wd.tev[1], st));
                wd.timing = 1;
                wd.timing_gi = gi;
            }
            ++wd.direct_runs[gi];
            continue;
        }
        if (!wd.graph[gi]) {
            cudaStream_t cap, cap2;
            CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
            CK(cudaStreamCreateWithPriority(&cap2, cudaStreamNonBlocking, L().prio_hi));
            cudaGraph_t graph;
            CK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
            const long long l0 = L().launches;
            int rc = issue_wave(s, wi, step, cap, cap2);
            cudaError_t e = cudaStreamEndCapture(cap, &graph);
            cudaStreamDestroy(cap);
            cudaStreamDestroy(cap2);
            if (rc != FWI_OK) return rc;
            if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture", __LINE__);
            wd.graph_kernels[gi] = L().launches - l0;
            L().launches = l0;  // counted when replayed
            e = cudaGraphInstantiate(&wd.graph[gi], graph, cudaGraphInstantiateFlagUseNodePriority);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate", __LINE__);
            CK(cudaGraphUpload(wd.graph[gi], st));  // outside the timed replay
        }
        const bool timed = wd.t_graph[gi] == 0.f;
        if (timed) CK(cudaEventRecord(wd.tev[0], st));
        CK(cudaGraphLaunch(wd.graph[gi], st));
        if (timed) {
            CK(cudaEventRecord(wd.tev[1], st));
            wd.timing = 2;
            wd.timing_gi = gi;
        }
        L().launches += wd.graph_kernels[gi];
    }
    if (s->obs_pending) {
        CK(cudaStreamWaitEvent(st, s->obs_ready, 0));
        s->obs_pending = false;
    }
    // per-shot misfits (FP64) in shot order
    std::vector<double> mis_tr(s->ntr);
    if (s->ntr) CK(cudaMemcpyAsync(mis_tr.data(), s->d_mis_tr.p, s->ntr * 8, cudaMemcpyDeviceToHost, st));
    if (grad && step == 1) {
        const size_t n = (size_t)D.ny * D.nx_model * 4;
        const bool dev = is_device_ptr(grad);
        float* dg = dev ? grad : s->d_grad.as<float>();
        if (!dev) CK(cudaMemcpyAsync(dg, grad, n, cudaMemcpyHostToDevice, st));
        LK(launch_finalize(dg, s->d_G.as<double>(), D.ny, D.nx_model, D.numtasks,
                           s->d_water.p ? s->d_water.as<int>() : nullptr, st));
        if (!dev) CK(cudaMemcpyAsync(grad, dg, n, cudaMemcpyDeviceToHost, st));
    }
    CK(cudaStreamSynchronize(st));
    // launch form: both timings known -> keep the faster one (a graph must
    // beat the direct launches by more than the 0.2 % run-to-run spread)
    for (auto& w : s->wdev) {
        auto& wd = *w;
        if (!wd.timing) continue;
        const int g2 = wd.timing_gi;
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, wd.tev[0], wd.tev[1]));
        if (wd.timing == 2) {
            wd.t_graph[g2] = ms;
        } else if (wd.recheck[g2]) {
            wd.t_direct[g2] = std::min(wd.t_direct[g2], ms);
            wd.recheck[g2] = false;
            wd.rechecked[g2] = true;
        } else {
            wd.t_direct[g2] = ms;
        }
        wd.timing = 0;
        if (wd.t_direct[g2] > 0.f && wd.t_graph[g2] > 0.f && wd.graph[g2] && !(D.flags & FWI_SURVEY_GRAPH)) {
            if (wd.t_graph[g2] > 1.002f * wd.t_direct[g2]) {
                CK(cudaGraphExecDestroy(wd.graph[g2]));
                wd.graph[g2] = nullptr;
                wd.direct_only[g2] = true;
            } else if (!wd.rechecked[g2]) {
                wd.recheck[g2] = true;  // the next run: direct launches once more
            }
        }
    }
    double tot = 0.0;
    bool finite = true;
    for (int i = 0; i < D.nshots; ++i) {
        double m = 0.0;
        for (int t = s->tr_off[i]; t < s->tr_off[i + 1]; ++t) m += mis_tr[t];
        if (!std::isfinite(m)) finite = false;
        tot += s->mw[i] * m;
    }
    if (misfit) *misfit += tot;
    if (!finite) return fail(FWI_ERR_NONFINITE, "non-finite misfit (the time step may violate the CFL limit)");
    return FWI_OK;
}

int fwi_survey_grad_device(fwi_survey* s, const double** ptr) {
    if (!s || !ptr) return fail(FWI_ERR_STATE, "null argument");
    *ptr = s->d_G.as<double>();
    return FWI_OK;
}

int fwi_survey_get_stack(fwi_survey* s, double* out) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    if (!s || !out) return fail(FWI_ERR_STATE, "null argument");
    const size_t n = (size_t)s->desc.ny * s->desc.nx_model * sizeof(double);
    CK(cudaMemcpyAsync(out, s->d_G.p, n, cudaMemcpyDeviceToHost, stream()));
    CK(cudaStreamSynchronize(stream()));
    return FWI_OK;
}

int fwi_survey_get_synthetic(fwi_survey* s, int shot, float* out) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    if (!s || !out) return fail(FWI_ERR_STATE, "null argument");
    if (shot < 0 || shot >= s->desc.nshots) return fail(FWI_ERR_ARG, "shot index out of range");
    const size_t n = (size_t)(s->tr_off[shot + 1] - s->tr_off[shot]) * s->desc.nt * 4;
    if (n)
        CK(cudaMemcpyAsync(out, s->d_synth.as<float>() + (size_t)s->tr_off[shot] * s->desc.nt, n,
                           cudaMemcpyDeviceToHost, stream()));
    CK(cudaStreamSynchronize(stream()));
    return FWI_OK;
}

int fwi_survey_step_bytes(fwi_survey* s, double* bytes) {
    if (!s || !bytes) return fail(FWI_ERR_STATE, "null argument");
    double b = 0.0;
    for (int sh : s->waves[0]) b += step_bytes_shot(s->lays[sh].ny, s->lays[sh].nx, s->lays[sh].dn);
    *bytes = b;
    return FWI_OK;
}

int fwi_survey_two_step_bytes(fwi_survey* s, double* per_step, double* tiles_per_pass) {
    if (!s || s->wdev.empty()) return fail(FWI_ERR_STATE, "survey not prepared");
    double b = 0.0;
    for (int sh : s->waves[0]) b += step_bytes_shot(s->lays[sh].ny, s->lays[sh].nx, s->lays[sh].dn);
    // a two-step tile reads p_n, p_{n-1}, c2 and writes p_{n+1}, p_{n+2} once
    // per cell and pass: 20 B for two steps instead of 2 x 16 B
    const double cells = s->wdev[0]->n_ff ? s->wdev[0]->fus_cells : 0.0;
    if (per_step) *per_step = b - 6.0 * cells;
    if (tiles_per_pass) *tiles_per_pass = 20.0 * cells;
    return FWI_OK;
}

int fwi_survey_tuning(fwi_survey* s, int* wave_shots, int* band_rows) {
    if (!s) return fail(FWI_ERR_STATE, "null survey");
    if (wave_shots) *wave_shots = s->wave;
    if (band_rows) *band_rows = s->band;
    return FWI_OK;
}

int fwi_survey_tiles(fwi_survey* s, int* tile_kernel, int* tile_rows, int* cand, float* times, int* ncand) {
    if (!s || s->wdev.empty()) return fail(FWI_ERR_STATE, "survey not prepared");
    const bool two = s->wdev[0]->n_ff > 0;
    if (tile_kernel) *tile_kernel = two ? s->tile_var + 1 : 0;
    if (tile_rows) *tile_rows = two ? s->tile_band : 0;
    if (ncand) *ncand = NTB;
    for (int c = 0; c < NTB; ++c) {
        if (cand) cand[c] = TILE_BANDS[c];
        if (times)
            for (int v = 0; v < 2; ++v) times[v * NTB + c] = s->tune_ms.empty() ? -1.f : s->tune_ms[v * NTB + c];
    }
    if (cand && s->desc.tile_rows > 0) cand[0] = s->desc.tile_rows;
    return FWI_OK;
}

int fwi_survey_edge_tiles(fwi_survey* s, int* edge_rows, int* cand, float* times, int* ncand) {
    if (!s || s->wdev.empty()) return fail(FWI_ERR_STATE, "survey not prepared");
    if (edge_rows) *edge_rows = s->wdev[0]->n_ff > 0 ? s->tile_eband : 0;
    if (ncand) *ncand = NEB;
    for (int c = 0; c < NEB; ++c) {
        if (cand) cand[c] = EDGE_BANDS[c];
        if (times) times[c] = s->tune_ems.empty() ? -1.f : s->tune_ems[c];
    }
    return FWI_OK;
}

int fwi_survey_stepping(fwi_survey* s, int* form, float* two_step_ms, float* single_ms, float* fused_ms) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    if (!s || s->wdev.empty()) return fail(FWI_ERR_STATE, "survey not prepared");
    if (form) *form = s->wdev[0]->n_ff > 0 ? 1 : (s->fused ? 2 : 0);
    if (two_step_ms) *two_step_ms = s->tune_two_ms;
    if (single_ms) *single_ms = s->tune_single_ms;
    if (fused_ms) *fused_ms = s->tune_fused_ms;
    return FWI_OK;
}

int fwi_survey_launch_form(fwi_survey* s, int step, int* form, float* direct_ms, float* graph_ms) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    if (!s || s->wdev.empty()) return fail(FWI_ERR_STATE, "survey not prepared");
    if (step != 1 && step != 2) return fail(FWI_ERR_ARG, "step must be 1 or 2");
    const auto& wd = *s->wdev[0];
    const int gi = step == 1 ? 0 : 1;
    if (form) {
        if (s->desc.flags & FWI_SURVEY_NO_GRAPH) *form = 2;
        else if (wd.direct_only[gi]) *form = 2;
        else if (wd.t_graph[gi] > 0.f) *form = 1;
        else *form = 0;
    }
    if (direct_ms) *direct_ms = wd.t_direct[gi];
    if (graph_ms) *graph_ms = wd.t_graph[gi];
    return FWI_OK;
}

int fwi_survey_recompute(fwi_survey* s, int* segment_steps, int* segments) {
    if (!s) return fail(FWI_ERR_STATE, "null survey");
    if (segment_steps) *segment_steps = s->rc_C;
    if (segments) *segments = s->rc_J;
    return FWI_OK;
}

int fwi_survey_time_steps(fwi_survey* s, int steps) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    if (!s) return fail(FWI_ERR_STATE, "null survey");
    return time_wave0_steps(s, steps, nullptr);
}

}  // extern "C"

namespace {
// `steps` forward steps of the first wave: two-step passes where the wave has
// two-step tiles (an even number of them, so that the state stays in pair 0)
// and single steps for the rest; single_only: single steps only.
int time_wave0_steps(fwi_survey* s, int steps, float* ms, bool single_only) {
    const auto& D = s->desc;
    auto& wd = *s->wdev[0];
    StepSet ps;
    ps.pm = base_params(D.acc, D.dt, D.store_snap, D.snap_form, D.grad_form, s->d_fA.as<float>(), s->d_fB.as<float>());
    ps.pm.items = wd.items_if.as<WorkItem>();
    ps.pm.nitems = wd.n_if;
    ps.pm.shots = wd.shots_f.as<ShotDev>();
    ps.pm.srcs = wd.src_f.as<SrcEnt>();
    ps.pm.recs = wd.recs.as<RecEnt>();
    ps.pm.record = 1;
    ps.pb = ps.pm;
    ps.pb.items = wd.items_bf.as<WorkItem>();
    ps.pb.nitems = wd.n_bf;
    ps.pb.nstrip = wd.n_strip;
    ps.kstrip = wd.kstrip;
    ps.fused = s->fused;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (ms) {
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        CK(cudaEventRecord(e0, stream()));
    }
    // pairs of steps as two-step passes when the wave has two-step tiles
    // (an even number of them, so that the state stays in pair 0)
    const TwoStep tw = two_step_set(ps, 0, wd.items_ff, wd.n_ff, wd.n_core, wd.items_lf, wd.n_lf, s->tile_var);
    const int npass = (wd.n_ff && D.nt >= 3 && !single_only) ? (steps / 4) * 2 : 0;
    // (in runs that stay inside the time axis: steps 2..nt)
    for (int done = 0, pair = 0; done < npass;) {
        const int n = std::min(npass - done, (D.nt - 1) / 2);
        TRY(two_step_run(D.acc, 0, tw, 2, n, nullptr, pair, stream(), L().aux));
        pair ^= n & 1;
        done += n;
    }
    for (int i = 2 * npass; i < steps; ++i) {
        const int k = 2 + (i % (D.nt - 1));
        set_step(ps, k, -1);
        TRY(step_fork_join(D.acc, 0, ps, stream(), L().aux));
    }
    if (ms) {
        CK(cudaEventRecord(e1, stream()));
        CK(cudaEventSynchronize(e1));
        CK(cudaEventElapsedTime(ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    return FWI_OK;
}
}  // namespace

extern "C" {

int fwi_misfit_gradient_batch(const fwi_survey_desc* desc, const float* lambda, int step, float* Misfit, float* Grad) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    TRY(ensure_init());
    if (!desc || !lambda) return fail(FWI_ERR_ARG, "null argument");
    if (desc->nshots < 1 || !desc->shots) return fail(FWI_ERR_ARG, "nshots must be >= 1");
    // plan key: the geometry (sizes, indices, weights, forms, tuning), not the
    // time axis -- the line search of FWI.f90:225-227 recomputes dt and nt from
    // every trial model (calculate_misfit_gradient.f90:198-203), which only
    // moves the survey to a new time axis (fwi_survey_set_time)
    std::string key;
    auto add = [&](const void* p, size_t n) { key.append(reinterpret_cast<const char*>(p), n); };
    fwi_survey_desc k0 = *desc;
    k0.shots = nullptr;
    k0.water_rows = nullptr;
    k0.dt = 0.f;
    k0.nt = 0;
    add(&k0, sizeof k0);
    for (int i = 0; i < desc->nshots; ++i) {
        const fwi_shot& sh = desc->shots[i];
        add(&sh.x0, sizeof(int) * 4);
        add(&sh.grad_weight, sizeof(double) * 2);
        if (sh.num_sou > 0 && sh.nxSou && sh.nySou) { add(sh.nxSou, 4 * sh.num_sou); add(sh.nySou, 4 * sh.num_sou); }
        if (sh.num_rec > 0 && sh.nxRec && sh.nyRec) { add(sh.nxRec, 4 * sh.num_rec); add(sh.nyRec, 4 * sh.num_rec); }
    }
    if (desc->water_rows) add(desc->water_rows, 4 * desc->nx_model);
    BatchPlan& bp = batch_plan();
    fwi_survey* s = nullptr;
    if (!bp.s || bp.key != key) {
        bp.release();  // the previous geometry's buffers first
        fwi_survey* ns = nullptr;
        TRY(fwi_survey_create(desc, &ns));
        bp.s = ns;
        bp.key = key;
        ++bp.plans;
        s = ns;
    } else {
        s = bp.s;
        if (desc->nt != s->desc.nt || desc->dt != s->desc.dt) {
            // a new time axis: the sources and data below are uploaded at the new length
            TRY(fwi_survey_set_time(s, desc->dt, desc->nt, nullptr, nullptr));
        }
        // this call's sources and observed data; copies whose host and
        // device ranges both continue the previous one are merged (callers
        // that pack all shots' data in one array get one copy per array)
        cudaStream_t st = stream();
        struct Run {
            const char* h = nullptr;
            char* d = nullptr;
            size_t n = 0;
        } rs, ro;
        auto put = [&](Run& r, const void* h, void* d, size_t n) -> int {
            if (r.n && static_cast<const char*>(h) == r.h + r.n && static_cast<char*>(d) == r.d + r.n) {
                r.n += n;
                return FWI_OK;
            }
            if (r.n) CK(cudaMemcpyAsync(r.d, r.h, r.n, cudaMemcpyHostToDevice, st));
            r.h = static_cast<const char*>(h);
            r.d = static_cast<char*>(d);
            r.n = n;
            return FWI_OK;
        };
        size_t so = 0, to = 0;
        const size_t nt = desc->nt;
        for (int i = 0; i < desc->nshots; ++i) {
            const fwi_shot& sh = desc->shots[i];
            if (sh.num_sou && sh.src)
                TRY(put(rs, sh.src, s->d_src.as<float>() + so, nt * sh.num_sou * 4));
            else if (sh.num_sou)
                CK(cudaMemsetAsync(s->d_src.as<float>() + so, 0, nt * sh.num_sou * 4, st));
            if (sh.num_rec && sh.obs)
                TRY(put(ro, sh.obs, s->d_obs.as<float>() + to, nt * sh.num_rec * 4));
            else if (sh.num_rec)
                CK(cudaMemsetAsync(s->d_obs.as<float>() + to, 0, nt * sh.num_rec * 4, st));
            so += nt * sh.num_sou;
            to += nt * sh.num_rec;
        }
        if (rs.n) CK(cudaMemcpyAsync(rs.d, rs.h, rs.n, cudaMemcpyHostToDevice, st));
        if (ro.n) {
            // the observed data: first read by the misfit, after the forward
            // pass, so they go on the copy stream beside it (ordered after
            // the work already on the stream)
            cudaStream_t sc = L().copy_in;
            CK(cudaEventRecord(s->obs_ready, st));
            CK(cudaStreamWaitEvent(sc, s->obs_ready, 0));
            CK(cudaMemcpyAsync(ro.d, ro.h, ro.n, cudaMemcpyHostToDevice, sc));
            CK(cudaEventRecord(s->obs_ready, sc));
            s->obs_pending = true;
        }
    }
    TRY(fwi_survey_set_lambda(s, lambda));
    double m = 0.0;
    const int rc = fwi_survey_run(s, step, &m, step == 1 ? Grad : nullptr);
    if (Misfit) *Misfit = *Misfit + (float)m;
    return rc;
}

int64_t fwi_batch_plans(void) { return batch_plan().plans; }

int fwi_batch_survey(fwi_survey** s) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    if (!s) return fail(FWI_ERR_ARG, "null argument");
    *s = batch_plan().s;
    return FWI_OK;
}

int fwi_batch_release(void) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    batch_plan().release();
    return FWI_OK;
}

}  // extern "C"

// ===========================================================================
// forward traces without device allocation
// ===========================================================================
//
// Some callers cannot call cudaMalloc: code that runs inside a framework
// which owns the device memory pool (a raw cudaMalloc synchronises the
// device and sits outside the pool's budget), and latency-critical code paths
// that must not allocate once they are set up.  For them the forward
// propagation of one shot can run with all of its working state (wavefields,
// c2, CPML memory variables, work lists) in the fixed array below, which
// every GPU that loads this library holds until the process exits.

namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = 16u << 20;  // 16 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch, looked up once per device.  In host
// code the symbol itself is only a host-side stand-in, so the kernels get
// this address instead.
constexpr int NOALLOC_MAX_DEVICES = 64;
void* g_noalloc_addr[NOALLOC_MAX_DEVICES] = {nullptr};

int noalloc_scratch(void** out) {
    const int dev = L().device;  // current on this thread (ensure_init)
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return fail(FWI_ERR_ARG, "device index too large");
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __LINE__);
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return FWI_OK;
}

}  // namespace

extern "C" int fwi_solver_forward_noalloc(int NumSou, int NumRec, const int* nxSou, const int* nySou,
                                          const int* nxRec, const int* nyRec, const float* S_dev, float d, float dt,
                                          int ny, int nx, const float* ctmp_dev, int nt, float* Rec_point_dev) {
    std::lock_guard<std::recursive_mutex> g(L().mu);
    TRY(ensure_init());
    const int acc = L().acc, dpml = L().dpml;
    TRY(validate_common(ny, nx, acc, dpml, nt, 1));
    if (NumSou < 0 || NumRec < 0) return fail(FWI_ERR_ARG, "NumSou/NumRec must be >= 0");
    if (!(d > 0.f) || !(dt > 0.f)) return fail(FWI_ERR_ARG, "d and dt must be positive");
    if (!ctmp_dev || (NumRec > 0 && (!Rec_point_dev || !nxRec || !nyRec)) ||
        (NumSou > 0 && (!S_dev || !nxSou || !nySou)))
        return fail(FWI_ERR_ARG, "null argument");
    const Layout l = make_layout(ny, nx, acc, dpml);
    ShotGeom geo;
    geo.nx = nx;
    geo.nxS.assign(nxSou, nxSou + NumSou);
    geo.nyS.assign(nySou, nySou + NumSou);
    geo.nxR.assign(nxRec, nxRec + NumRec);
    geo.nyR.assign(nyRec, nyRec + NumRec);
    TRY(validate_geometry(geo, l, 1));
    std::vector<ShotGeom> geoms{geo};
    std::vector<Layout> lays{l};
    Lists lists = build_lists(geoms, lays, 64);
    std::vector<float> fA, fB;
    pml_factors(acc, dpml, dt, d, fA, fB);

    // carve the scratch: eight fields, CPML factors, shot descriptor, lists
    const size_t field = (size_t)l.nyt * l.pitch * sizeof(float);
    size_t off = 0;
    auto carve = [&](size_t bytes) {
        const size_t at = off;
        off += (bytes + 255) / 256 * 256;
        return at;
    };
    size_t o_fld[8];
    for (auto& o : o_fld) o = carve(field);
    const size_t o_fA = carve(fA.size() * 4), o_fB = carve(fB.size() * 4), o_shot = carve(sizeof(ShotDev));
    const size_t o_im = carve(lists.int_fwd.size() * sizeof(WorkItem)), o_bm = carve(lists.bnd_fwd.size() * sizeof(WorkItem));
    const size_t o_src = carve(lists.src_fwd.size() * sizeof(SrcEnt)), o_rec = carve(lists.recs.size() * sizeof(RecEnt));
    if (off > NOALLOC_SCRATCH_BYTES) {
        char buf[256];
        snprintf(buf, sizeof buf,
                 "grid too large for the allocation-free solver: needs %zu bytes of scratch, the fixed limit is %zu "
                 "(use fwi_solver_acoustic_ss)",
                 off, NOALLOC_SCRATCH_BYTES);
        return fail(FWI_ERR_ARG, buf);
    }
    void* base = nullptr;
    TRY(noalloc_scratch(&base));
    unsigned char* sb = reinterpret_cast<unsigned char*>(base);
    cudaStream_t st = stream();

    // the array keeps the previous call's contents: clear the state that must start at zero
    CK(cudaMemsetAsync(sb, 0, o_fA, st));
    float* fld[8];
    for (int i = 0; i < 8; ++i) fld[i] = reinterpret_cast<float*>(sb + o_fld[i]);
    LK(launch_build_c2(fld[2], l.nyt, l.pitch, l.off, l.dn, ny, nx, ctmp_dev, ny, 0, 0, dt * dt, d * d, st));
    if (NumRec > 0) CK(cudaMemsetAsync(Rec_point_dev, 0, (size_t)nt * NumRec * sizeof(float), st));

    ShotDev sd{};
    sd.pf[0] = fld[0];
    sd.pf[1] = fld[1];
    sd.c2 = fld[2];
    sd.phx = fld[3];
    sd.chx = fld[4];
    sd.phy = fld[5];
    sd.chy = fld[6];
    sd.phy2 = fld[7];
    sd.srcv = S_dev;
    sd.rec = Rec_point_dev;
    sd.ny = l.ny; sd.nx = l.nx; sd.nyt = l.nyt; sd.nxt = l.nxt; sd.off = l.off; sd.pitch = l.pitch;
    sd.ntiles = l.ntiles; sd.dn = l.dn; sd.sl = l.sl; sd.sr = l.sr; sd.nt = nt; sd.nrec = NumRec;
    auto put = [&](size_t at, const void* src, size_t bytes) -> int {
        if (bytes) CK(cudaMemcpyAsync(sb + at, src, bytes, cudaMemcpyHostToDevice, st));
        return FWI_OK;
    };
    TRY(put(o_fA, fA.data(), fA.size() * 4));
    TRY(put(o_fB, fB.data(), fB.size() * 4));
    TRY(put(o_shot, &sd, sizeof sd));
    TRY(put(o_im, lists.int_fwd.data(), lists.int_fwd.size() * sizeof(WorkItem)));
    TRY(put(o_bm, lists.bnd_fwd.data(), lists.bnd_fwd.size() * sizeof(WorkItem)));
    TRY(put(o_src, lists.src_fwd.data(), lists.src_fwd.size() * sizeof(SrcEnt)));
    TRY(put(o_rec, lists.recs.data(), lists.recs.size() * sizeof(RecEnt)));

    StepSet ps;
    ps.pm = base_params(acc, dt, nt + 1, FWI_SNAP_F32, FWI_GRAD_F32, reinterpret_cast<float*>(sb + o_fA),
                        reinterpret_cast<float*>(sb + o_fB));
    ps.pm.items = reinterpret_cast<WorkItem*>(sb + o_im);
    ps.pm.nitems = (int)lists.int_fwd.size();
    ps.pm.shots = reinterpret_cast<ShotDev*>(sb + o_shot);
    ps.pm.srcs = reinterpret_cast<SrcEnt*>(sb + o_src);
    ps.pm.recs = reinterpret_cast<RecEnt*>(sb + o_rec);
    ps.pm.record = 1;
    ps.pb = ps.pm;
    ps.pb.items = reinterpret_cast<WorkItem*>(sb + o_bm);
    ps.pb.nitems = (int)lists.bnd_fwd.size();
    ps.pb.nstrip = lists.nstrip;
    ps.kstrip = lists.kstrip;
    TRY(run_time_loop(acc, 0, nt, nt + 1, 0, false, ps, st, L().aux));
    LK(launch_rec_last(Rec_point_dev, nt, NumRec, st));
    CK(cudaStreamSynchronize(st));
    return FWI_OK;
}
