// agb_api.cu -- host side of the C ABI declared in include/agb.h.
//
// Owns the level hierarchy (Operator<Node>::define / MLLinOp coarsening), the
// device buffers, and the cycle driver that restates AMReX MLMG as Alamo
// configures it (Solver/Nonlocal/Linear.H:255-290): F-cycles for the first
// max_fmg_iter iterations then V-cycles, pre/post smoothing by Fsmooth,
// BiCGStab bottom solve, ||r||_inf stopping test.  Every kernel is queued on the
// operator's stream; a whole iteration (cycle + update + residual norm) is
// captured once into a CUDA graph and replayed, with one 8-byte read-back per
// iteration for the convergence test.
//
// Mixed precision (AGB_PREC_MIXED): FP32 cycles solve the correction equation
// of an FP64 iterative refinement.  FP64 is kept for the outer residual
// b - A x, the accumulation of x and the coarsest-level solve.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/agb.h"
#include "agb_internal.h"

using namespace agb;

namespace {

thread_local std::string g_err;

agb_status fail(agb_status s, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return s;
}

#define CK(call)                                                                                      \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return fail(AGB_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                           __FILE__, __LINE__);                                       \
    } while (0)

#define TRY(...)                         \
    do {                                 \
        agb_status s_ = (__VA_ARGS__);   \
        if (s_ != AGB_OK) return s_;     \
    } while (0)

struct Level {
    LevelDesc L;
    double* ddw64 = nullptr;
    float* ddw32 = nullptr;
    double* diag64 = nullptr;
    double* dinv64 = nullptr;
    float* dinv32 = nullptr;
    double *cor64 = nullptr, *res64 = nullptr, *rescor64 = nullptr, *hold64 = nullptr, *tmp64 = nullptr;
    float *cor32 = nullptr, *res32 = nullptr, *rescor32 = nullptr, *hold32 = nullptr, *tmp32 = nullptr;
};

bool g_attr_done = false;

}  // namespace

namespace agb {
long long& launch_counter()
{
    static long long n = 0;
    return n;
}
void set_error(const char* msg) { g_err = msg ? msg : ""; }
bool pdl_enabled()
{
    static bool v = [] {
        const char* s = getenv("AGB_PDL");
        return s && s[0] == '1';
    }();
    return v;
}
int sm_count()
{
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return 1;
    }
    int v = __atomic_load_n(&cache[dev], __ATOMIC_RELAXED);
    if (v > 0) return v;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v < 1) {
        cudaGetLastError();
        return 1;
    }
    __atomic_store_n(&cache[dev], v, __ATOMIC_RELAXED);
    return v;
}
}  // namespace agb

struct agb_op_s {
    int sym = 0, nc = 2;
    int n[3] = {0, 0, 0}, per[3] = {0, 0, 0};
    double dx[3] = {0, 0, 0};
    bool uniform = false;
    double omega = 2.0 / 3.0;
    BCTable bc;
    bool bc_set = false, model_set = false, prepared = false, f32_ready = false;
    std::vector<Level> lev;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    double* d_slots = nullptr;   // 16 x 8 bytes of reduction slots
    double* h_slots = nullptr;   // pinned mirror
    double* bottom_work = nullptr;
    double* bottom_A = nullptr;   // dense coarsest-level operator (small bottom levels)
    float* bottom_inv32 = nullptr;   // its inverse for the FP32 cycles (exact coarsest solve)
    int* bottom_inv_ok = nullptr;    // device flag: the inverse exists
    int* d_ret = nullptr;
    char* stage = nullptr;       // bounded staging buffer for pageable host copies
    size_t stage_bytes = 0;
    char* dma = nullptr;         // whole-field staging buffer for pinned host copies (grown on demand)
    size_t dma_bytes = 0;
    double *nw_dw = nullptr, *nw_u0 = nullptr, *nw_F0 = nullptr;   // Newton work fields, kept across calls
    int pageable_ok = 0;         // device can read pageable host memory directly
    std::vector<void*> allocs;

    template <typename T> agb_status alloc(T** p, size_t count)
    {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
        if (e != cudaSuccess) return fail(AGB_NOMEM, "cudaMalloc(%zu bytes): %s", count * sizeof(T), cudaGetErrorString(e));
        e = cudaMemsetAsync(q, 0, std::max<size_t>(count, 1) * sizeof(T), st);
        if (e != cudaSuccess) return fail(AGB_CUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
        allocs.push_back(q);
        *p = (T*)q;
        return AGB_OK;
    }
};

struct agb_solver_s {
    agb_op op = nullptr;
    agb_solver_params p;
    double *x64 = nullptr, *b64 = nullptr, *F0 = nullptr, *dw = nullptr;
    float *rhs32 = nullptr, *sol32 = nullptr;
    cudaGraphExec_t g64 = nullptr, g32 = nullptr;
    int g64_fcycle = -1, g32_fcycle = -1;   // cycle kind each graph holds
    long long g64_kernels = 0, g32_kernels = 0;
    long long replayed = 0;                  // kernels executed through graph replays
    // inner FP32 GCR of the mixed solve (params.krylov > 0): directions, their
    // images, the inner residual, device scalars, the preconditioner's graph
    std::vector<float*> kZ, kW;
    float* kr = nullptr;
    double* kdots = nullptr;
    cudaGraphExec_t gpre = nullptr;
    long long gpre_kernels = 0;
    // learned correction (agb_solver_set_learned): the network, the
    // acceptance threshold and the count of consecutive rejections that
    // switches it off for the rest of a solve; per-solve statistics
    agb_learned net = nullptr;
    double learned_min_gain = 0.01;
    int learned_max_fail = 2;
    bool learned_on = false;
    int learned_tried = 0, learned_kept = 0, learned_fails = 0;
};

// ---------------------------------------------------------------------------
// host <-> device field movement
// ---------------------------------------------------------------------------
namespace {

// Device fields may still be written by work the caller queued on the legacy
// default stream (where torch and most callers queue): wait for it before
// the operator's non-blocking stream touches them.
agb_status caller_ready(int mem)
{
    if (mem == AGB_MEM_DEVICE) CK(cudaStreamSynchronize(cudaStreamLegacy));
    return AGB_OK;
}

// Pinned host memory is read (written) in place by the import (export)
// kernel through its mapped device address.  On GB300 that moves a field at
// the host link's rate every time (a 2.85 GB Matrix4 field: 14.7 ms), while
// a copy-engine transfer of the same field ran at 25-45 GB/s for its first
// pass after a stretch of device-only work (14.6-106 ms measured), so the
// copy engine is only the fallback for pinned memory without a mapping.
const void* mapped_host(const void* p, int mem)
{
    if (mem == AGB_MEM_DEVICE) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

bool pinned_host(const void* p, int mem)
{
    if (mem == AGB_MEM_DEVICE) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

agb_status dma_buffer(agb_op op, size_t bytes, char** out)
{
    if (bytes > op->dma_bytes) {
        if (op->dma) {
            CK(cudaStreamSynchronize(op->st));
            cudaFree(op->dma);
            op->dma = nullptr;
            op->dma_bytes = 0;
        }
        if (cudaMalloc(&op->dma, bytes) != cudaSuccess) {
            cudaGetLastError();
            return fail(AGB_NOMEM, "cudaMalloc(%zu bytes) for the host copy", bytes);
        }
        op->dma_bytes = bytes;
    }
    *out = op->dma;
    return AGB_OK;
}

bool directly_readable(agb_op op, const void* p, int mem)
{
    if (mem == AGB_MEM_DEVICE) return true;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return op->pageable_ok != 0;
    }
    if (a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return true;
    return op->pageable_ok != 0;
}

template <typename TD, typename TS>
agb_status upload(agb_op op, const LevelDesc& L, int ncomp, bool aos, const TS* src, int mem, TD* dst)
{
    if (!src) return fail(AGB_BADARG, "null input field");
    TRY(caller_ready(mem));
    const int nk = L.n[2] + 1;
    if (const TS* m = (const TS*)mapped_host(src, mem)) {
        launch_import<TD, TS>(op->st, L, ncomp, m, dst, aos, 0, L.nn[2], false);
        CK(cudaGetLastError());
        return AGB_OK;
    }
    if (pinned_host(src, mem)) {
        const size_t bytes = sizeof(TS) * (size_t)(L.n[0] + 1) * (L.n[1] + 1) * nk * ncomp;
        char* buf = nullptr;
        TRY(dma_buffer(op, bytes, &buf));
        CK(cudaMemcpyAsync(buf, src, bytes, cudaMemcpyHostToDevice, op->st));
        launch_import<TD, TS>(op->st, L, ncomp, (const TS*)buf, dst, aos, 0, L.nn[2], false);
        CK(cudaGetLastError());
        return AGB_OK;
    }
    if (directly_readable(op, src, mem)) {
        launch_import<TD, TS>(op->st, L, ncomp, src, dst, aos, 0, L.nn[2], false);
        CK(cudaGetLastError());
        return AGB_OK;
    }
    const size_t planeN = (size_t)(L.n[0] + 1) * (L.n[1] + 1);
    const size_t per_plane = planeN * ncomp * sizeof(TS);
    int kc = (int)std::max<size_t>(1, op->stage_bytes / per_plane);
    for (int k0 = 0; k0 < L.nn[2]; k0 += kc) {
        const int kk = std::min(kc, L.nn[2] - k0);
        TS* stg = (TS*)op->stage;
        if (aos) {
            CK(cudaMemcpyAsync(stg, src + (size_t)k0 * planeN * ncomp, planeN * ncomp * kk * sizeof(TS),
                               cudaMemcpyHostToDevice, op->st));
        } else {
            for (int c = 0; c < ncomp; c++)
                CK(cudaMemcpyAsync(stg + (size_t)c * planeN * kk, src + (size_t)c * planeN * nk + (size_t)k0 * planeN,
                                   planeN * kk * sizeof(TS), cudaMemcpyHostToDevice, op->st));
        }
        launch_import<TD, TS>(op->st, L, ncomp, stg, dst, aos, k0, kk, true);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(op->st));
    }
    return AGB_OK;
}

template <typename TD, typename TS>
agb_status download(agb_op op, const LevelDesc& L, int ncomp, bool aos, const TS* src, TD* dst, int mem)
{
    if (!dst) return fail(AGB_BADARG, "null output field");
    TRY(caller_ready(mem));
    const int nk = L.n[2] + 1;
    if (TD* m = (TD*)mapped_host(dst, mem)) {
        launch_export<TD, TS>(op->st, L, ncomp, src, m, aos, 0, nk, false);
        CK(cudaGetLastError());
        return AGB_OK;
    }
    if (pinned_host(dst, mem)) {
        const size_t bytes = sizeof(TD) * (size_t)(L.n[0] + 1) * (L.n[1] + 1) * nk * ncomp;
        char* buf = nullptr;
        TRY(dma_buffer(op, bytes, &buf));
        launch_export<TD, TS>(op->st, L, ncomp, src, (TD*)buf, aos, 0, nk, false);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(dst, buf, bytes, cudaMemcpyDeviceToHost, op->st));
        return AGB_OK;
    }
    if (directly_readable(op, dst, mem)) {
        launch_export<TD, TS>(op->st, L, ncomp, src, dst, aos, 0, nk, false);
        CK(cudaGetLastError());
        return AGB_OK;
    }
    const size_t planeN = (size_t)(L.n[0] + 1) * (L.n[1] + 1);
    const size_t per_plane = planeN * ncomp * sizeof(TD);
    int kc = (int)std::max<size_t>(1, op->stage_bytes / per_plane);
    for (int k0 = 0; k0 < nk; k0 += kc) {
        const int kk = std::min(kc, nk - k0);
        TD* stg = (TD*)op->stage;
        launch_export<TD, TS>(op->st, L, ncomp, src, stg, aos, k0, kk, true);
        CK(cudaGetLastError());
        if (aos) {
            CK(cudaMemcpyAsync(dst + (size_t)k0 * planeN * ncomp, stg, planeN * ncomp * kk * sizeof(TD),
                               cudaMemcpyDeviceToHost, op->st));
        } else {
            for (int c = 0; c < ncomp; c++)
                CK(cudaMemcpyAsync(dst + (size_t)c * planeN * nk + (size_t)k0 * planeN, stg + (size_t)c * planeN * kk,
                                   planeN * kk * sizeof(TD), cudaMemcpyDeviceToHost, op->st));
        }
        CK(cudaStreamSynchronize(op->st));
    }
    return AGB_OK;
}

int num_levels(const int n[3], int max_coarsening_level)
{
    int m[3] = {n[0], n[1], n[2]}, lev = 1;
    while (lev - 1 < max_coarsening_level) {
        bool ok = true;
        for (int d = 0; d < 3; d++)
            if (m[d] % 2 != 0 || m[d] / 2 < 2) ok = false;
        if (!ok) break;
        for (int d = 0; d < 3; d++) m[d] /= 2;
        lev++;
    }
    return lev;
}

agb_status check_level(agb_op op, int level)
{
    if (!op) return fail(AGB_BADARG, "null operator");
    if (level < 0 || level >= (int)op->lev.size()) return fail(AGB_BADARG, "level %d out of range", level);
    return AGB_OK;
}

agb_status ensure_f32(agb_op op)
{
    if (op->f32_ready) return AGB_OK;
    for (auto& lv : op->lev) {
        const size_t n3 = 3 * (size_t)lv.L.S;
        if (!lv.ddw32) TRY(op->alloc(&lv.ddw32, op->nc * (size_t)lv.L.S));
        if (!lv.dinv32) TRY(op->alloc(&lv.dinv32, n3));
        if (!lv.cor32) {
            TRY(op->alloc(&lv.cor32, n3));
            TRY(op->alloc(&lv.res32, n3));
            TRY(op->alloc(&lv.rescor32, n3));
            TRY(op->alloc(&lv.hold32, n3));
            TRY(op->alloc(&lv.tmp32, n3));
        }
        launch_convert<float, double>(op->st, lv.L, op->nc, lv.ddw64, lv.ddw32, 1.0);
        launch_recip<float>(op->st, lv.L, 3, lv.diag64, lv.dinv32);
    }
    // prepare() assembled the dense coarsest operator; the FP32 cycles take its inverse
    if (op->bottom_inv32)
        launch_bottom_invert(op->st, op->lev.back().L, op->bottom_A, op->bottom_inv32, op->bottom_inv_ok);
    CK(cudaGetLastError());
    op->f32_ready = true;
    return AGB_OK;
}

agb_status prepare(agb_op op);

// prepareForSolve for the mixed solve.  Its FP32 cycles read the FP32
// hierarchy only, so that is built in FP32 from the finest FP64 moduli:
// coefficients averaged and diagonals computed in FP32 (in FP64 those passes
// take ~14 ms at 257^3 on GB300, whose FP64 rate they are bound by).  The
// bottom level's FP64 moduli (converted), diagonal and dense operator are made
// as well, for the bottom solve reads those.  The finest level's FP64 moduli
// (SetModel) serve the FP64 residuals.  The FP64 hierarchy of the other
// levels is left stale (prepared = false) until an FP64 consumer calls
// prepare().
agb_status prepare_mixed(agb_op op)
{
    if (!op->model_set) return fail(AGB_STATE, "SetModel must be called before the operator is used");
    if (!op->bc_set) return fail(AGB_STATE, "SetBC must be called before the operator is used");
    for (auto& lv : op->lev) {
        const size_t n3 = 3 * (size_t)lv.L.S;
        if (!lv.ddw32) TRY(op->alloc(&lv.ddw32, op->nc * (size_t)lv.L.S));
        if (!lv.dinv32) TRY(op->alloc(&lv.dinv32, n3));
        if (!lv.cor32) {
            TRY(op->alloc(&lv.cor32, n3));
            TRY(op->alloc(&lv.res32, n3));
            TRY(op->alloc(&lv.rescor32, n3));
            TRY(op->alloc(&lv.hold32, n3));
            TRY(op->alloc(&lv.tmp32, n3));
        }
    }
    const size_t nl = op->lev.size();
    launch_convert<float, double>(op->st, op->lev[0].L, op->nc, op->lev[0].ddw64, op->lev[0].ddw32, 1.0);
    for (size_t l = 1; l < nl; l++)
        launch_average_ddw<float>(op->st, op->lev[l - 1].L, op->lev[l].L, op->lev[l - 1].ddw32, op->lev[l].ddw32,
                                  op->nc);
    for (auto& lv : op->lev) {
        launch_diagonal<float>(op->st, op->sym, lv.L, op->bc, lv.ddw32, lv.dinv32);
        launch_recip_inplace(op->st, lv.L, 3, lv.dinv32);
    }
    Level& bl = op->lev[nl - 1];
    if (nl > 1) launch_convert<double, float>(op->st, bl.L, op->nc, bl.ddw32, bl.ddw64, 1.0);
    launch_diagonal<double>(op->st, op->sym, bl.L, op->bc, bl.ddw64, bl.diag64);
    launch_recip<double>(op->st, bl.L, 3, bl.diag64, bl.dinv64);
    if (op->bottom_A)
        launch_bottom_assemble(op->st, op->sym, bl.L, op->bc, op->uniform, bl.ddw64, op->bottom_A);
    if (op->bottom_inv32) launch_bottom_invert(op->st, bl.L, op->bottom_A, op->bottom_inv32, op->bottom_inv_ok);
    CK(cudaGetLastError());
    op->prepared = false;
    op->f32_ready = true;
    return AGB_OK;
}

// MLMG::solve -> prepareForSolve on every call, for the solver's precision
agb_status prepare_for_solve(agb_solver s)
{
    agb_op op = s->op;
    op->prepared = false;
    return s->p.precision == AGB_PREC_MIXED ? prepare_mixed(op) : prepare(op);
}

// averageDownCoeffs + Diagonal(true) for every level (Operator.cpp:253-260)
agb_status prepare(agb_op op)
{
    if (!op->model_set) return fail(AGB_STATE, "SetModel must be called before the operator is used");
    if (!op->bc_set) return fail(AGB_STATE, "SetBC must be called before the operator is used");
    if (op->prepared) return AGB_OK;
    for (size_t l = 1; l < op->lev.size(); l++)
        launch_average_ddw<double>(op->st, op->lev[l - 1].L, op->lev[l].L, op->lev[l - 1].ddw64, op->lev[l].ddw64, op->nc);
    for (auto& lv : op->lev) {
        launch_diagonal<double>(op->st, op->sym, lv.L, op->bc, lv.ddw64, lv.diag64);
        launch_recip<double>(op->st, lv.L, 3, lv.diag64, lv.dinv64);
    }
    if (op->bottom_A)
        launch_bottom_assemble(op->st, op->sym, op->lev.back().L, op->bc, op->uniform, op->lev.back().ddw64,
                               op->bottom_A);
    CK(cudaGetLastError());
    op->prepared = true;
    op->f32_ready = false;
    return AGB_OK;
}

// ---------------------------------------------------------------------------
// cycle engine (MLMG restated), templated on the cycle arithmetic
// ---------------------------------------------------------------------------
template <typename T> struct Arr;
template <> struct Arr<double> {
    static double* cor(Level& l) { return l.cor64; }
    static double* res(Level& l) { return l.res64; }
    static double* rescor(Level& l) { return l.rescor64; }
    static double* hold(Level& l) { return l.hold64; }
    static double* tmp(Level& l) { return l.tmp64; }
    static const double* ddw(Level& l) { return l.ddw64; }
    static const double* dinv(Level& l) { return l.dinv64; }
    static void swap_res_rescor(Level& l) { std::swap(l.res64, l.rescor64); }
    static void swap_cor_hold(Level& l) { std::swap(l.cor64, l.hold64); }
};
template <> struct Arr<float> {
    static float* cor(Level& l) { return l.cor32; }
    static float* res(Level& l) { return l.res32; }
    static float* rescor(Level& l) { return l.rescor32; }
    static float* hold(Level& l) { return l.hold32; }
    static float* tmp(Level& l) { return l.tmp32; }
    static const float* ddw(Level& l) { return l.ddw32; }
    static const float* dinv(Level& l) { return l.dinv32; }
    static void swap_res_rescor(Level& l) { std::swap(l.res32, l.rescor32); }
    static void swap_cor_hold(Level& l) { std::swap(l.cor32, l.hold32); }
};

template <typename T> struct Engine {
    agb_op op;
    const agb_solver_params& p;
    typedef Arr<T> A;
    Level& lv(int l) { return op->lev[l]; }
    int bot() const { return (int)op->lev.size() - 1; }

    void sweep2(int l, T* x, const T* b)
    {
        Level& v = lv(l);
        launch_stencil<T>(op->st, op->sym, MODE_JACOBI, v.L, op->bc, op->uniform, A::ddw(v), x, b, A::dinv(v),
                          A::tmp(v), (T)op->omega, nullptr);
        launch_stencil<T>(op->st, op->sym, MODE_JACOBI, v.L, op->bc, op->uniform, A::ddw(v), A::tmp(v), b,
                          A::dinv(v), x, (T)op->omega, nullptr);
    }
    void smooth(int l, T* x, const T* b, int nsmooth)
    {
        for (int s = 0; s < nsmooth; s++) sweep2(l, x, b);
    }
    // x = 0, then Fsmooth: the first sweep of a zero guess is elementwise
    // (launch_jacobi_zero), the rest are stencil sweeps
    void smooth_from_zero(int l, T* x, const T* b, int nsmooth)
    {
        Level& v = lv(l);
        if (nsmooth <= 0) {
            launch_zero<T>(op->st, v.L, 3, x);
            return;
        }
        launch_jacobi_zero<T>(op->st, v.L, 3, A::tmp(v), b, A::dinv(v), (T)op->omega);
        launch_stencil<T>(op->st, op->sym, MODE_JACOBI, v.L, op->bc, op->uniform, A::ddw(v), A::tmp(v), b,
                          A::dinv(v), x, (T)op->omega, nullptr);
        for (int s = 1; s < nsmooth; s++) sweep2(l, x, b);
    }
    void residual(int l, const T* x, const T* b, T* r, void* slot)
    {
        Level& v = lv(l);
        launch_stencil<T>(op->st, op->sym, MODE_RESID, v.L, op->bc, op->uniform, A::ddw(v), x, b, nullptr, r, (T)0,
                          slot);
    }
    // The solve's fine-level residual and its max norm (into a zeroed slot).
    // A fully periodic box is singular (rigid translations) and the operator
    // is not conservative, so its left null vectors are constants only up to
    // discretisation error: the solve projects the right-hand side and every
    // fine residual (and, in the bottom solve, every Krylov residual and
    // operator application) to zero mean per component, and so finds u with
    // A u = b - c for a uniform body force c of the size of that error.
    void fine_residual(const T* x, const T* b, T* r, void* slot)
    {
        Level& v = lv(0);
        if (!v.L.singular()) return residual(0, x, b, r, slot);
        residual(0, x, b, r, nullptr);
        launch_remove_mean<T>(op->st, v.L, r, op->d_slots + 11, slot);
    }
    void bottom()
    {
        Level& v = lv(bot());
        if (op->bottom_A) {
            // the FP32 cycles of the mixed solve take the exact coarsest solve
            // when prepare_mixed made the inverse; the FP64 cycles keep MLMG's
            // BiCGStab bottom
            const bool exact = sizeof(T) == 4 && op->bottom_inv32 && op->f32_ready;
            launch_bottom_dense<T>(op->st, v.L, op->bottom_A, v.diag64, A::cor(v), A::res(v), p.bottom_max_iter,
                                   p.bottom_tol_rel, p.bottom_tol_abs, op->d_ret, p.bottom_smooth, p.final_smooth,
                                   op->omega, exact ? op->bottom_inv32 : nullptr, exact ? op->bottom_inv_ok : nullptr);
            return;
        }
        launch_bottom<T>(op->st, op->sym, v.L, op->bc, op->uniform, v.ddw64, v.diag64, A::cor(v), A::res(v),
                         op->bottom_work, p.bottom_max_iter, p.bottom_tol_rel, p.bottom_tol_abs, op->d_ret,
                         p.bottom_smooth, p.final_smooth, op->omega);
    }
    // MLMG::mgVcycle(amrlev = 0, mglev_top)
    void vcycle(int top)
    {
        const int b = bot();
        for (int l = top; l < b; l++) {
            Level& v = lv(l);
            smooth_from_zero(l, A::cor(v), A::res(v), p.pre_smooth);
            residual(l, A::cor(v), A::res(v), A::rescor(v), nullptr);
            launch_restriction<T>(op->st, v.L, lv(l + 1).L, A::rescor(v), A::res(lv(l + 1)), 3);
        }
        bottom();
        for (int l = b - 1; l >= top; l--) {
            Level& v = lv(l);
            launch_interpolation<T>(op->st, v.L, lv(l + 1).L, A::cor(v), A::cor(lv(l + 1)), false);
            smooth(l, A::cor(v), A::res(v), p.post_smooth);
        }
    }
    // MLMG::mgFcycle
    void fcycle()
    {
        const int b = bot();
        for (int l = 1; l <= b; l++)
            launch_restriction<T>(op->st, lv(l - 1).L, lv(l).L, A::res(lv(l - 1)), A::res(lv(l)), 3);
        bottom();
        for (int l = b - 1; l >= 0; l--) {
            Level& v = lv(l);
            launch_interpolation<T>(op->st, v.L, lv(l + 1).L, A::cor(v), A::cor(lv(l + 1)), true);
            residual(l, A::cor(v), A::res(v), A::rescor(v), nullptr);
            // The V-cycle's right-hand side is the residual of the interpolated
            // correction, and the interpolated correction is kept aside: swap
            // the buffers' roles instead of copying (res <-> rescor, cor <->
            // hold), add the V-cycle's correction into the kept one, and swap
            // back, so that cor holds the sum and every buffer has its role
            // again when the step ends (the captured graph replays from there).
            A::swap_res_rescor(v);
            A::swap_cor_hold(v);
            vcycle(l);
            launch_axpy<T>(op->st, v.L, 3, A::hold(v), A::cor(v), (T)1);
            A::swap_res_rescor(v);
            A::swap_cor_hold(v);
        }
    }
    void cycle(int iter)
    {
        if (iter < p.max_fmg_iter) fcycle();
        else vcycle(0);
    }
};

agb_status sync_read(agb_op op, double* out, int count)
{
    CK(cudaStreamSynchronize(op->st));
    for (int i = 0; i < count; i++) out[i] = op->h_slots[i];
    return AGB_OK;
}

double slot_as_double(const double* slots, int i) { return slots[i]; }
double slot_as_float(const double* slots, int i)
{
    float f;
    memcpy(&f, &slots[i], sizeof(float));
    return (double)f;
}

// One FP64 MLMG iteration on (x64, b64): cycle, x += cor, r = b - A x, ||r|| -> slot 0.
void iter64_body(agb_solver s, int iter)
{
    agb_op op = s->op;
    Engine<double> E{op, s->p};
    Level& v0 = op->lev[0];
    E.cycle(iter);
    launch_axpy<double>(op->st, v0.L, 3, s->x64, v0.cor64, 1.0);
    cudaMemsetAsync(op->d_slots, 0, sizeof(double), op->st);
    E.fine_residual(s->x64, s->b64, v0.res64, op->d_slots);
    cudaMemcpyAsync(op->h_slots, op->d_slots, sizeof(double), cudaMemcpyDeviceToHost, op->st);
}

// One FP32 inner iteration on (sol32, rhs32): cycle, sol += cor, res = rhs - A sol, ||res|| -> slot 1.
void iter32_body(agb_solver s, int iter)
{
    agb_op op = s->op;
    Engine<float> E{op, s->p};
    Level& v0 = op->lev[0];
    E.cycle(iter);
    launch_axpy<float>(op->st, v0.L, 3, s->sol32, v0.cor32, 1.0f);
    cudaMemsetAsync(op->d_slots + 1, 0, sizeof(double), op->st);
    E.fine_residual(s->sol32, s->rhs32, v0.res32, op->d_slots + 1);
    cudaMemcpyAsync(op->h_slots + 1, op->d_slots + 1, sizeof(double), cudaMemcpyDeviceToHost, op->st);
}

// Capture fn into a graph on the operator stream (F-cycle iterations only; a
// V-cycle iteration is launched directly).
template <class Fn> agb_status capture(agb_op op, cudaGraphExec_t* out, Fn fn)
{
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(op->st, cudaStreamCaptureModeThreadLocal));
    fn();
    cudaError_t e = cudaStreamEndCapture(op->st, &g);
    if (e != cudaSuccess) return fail(AGB_CUDA, "graph capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(AGB_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    return AGB_OK;
}

agb_status run_iter64(agb_solver s, int iter)
{
    agb_op op = s->op;
    const bool fc = iter < s->p.max_fmg_iter;
    if (s->p.use_graph) {
        // F-cycle and V-cycle iterations have different kernel sequences; the
        // graph holds whichever kind the solve is running now.
        if (s->g64 && s->g64_fcycle != (int)fc) {
            cudaGraphExecDestroy(s->g64);
            s->g64 = nullptr;
        }
        if (!s->g64) {
            const long long k0 = launch_counter();
            TRY(capture(op, &s->g64, [&] { iter64_body(s, fc ? 0 : s->p.max_fmg_iter); }));
            s->g64_kernels = launch_counter() - k0;
            launch_counter() = k0;
        }
        s->g64_fcycle = (int)fc;
        CK(cudaGraphLaunch(s->g64, op->st));
        s->replayed += s->g64_kernels;
    } else {
        iter64_body(s, iter);
        CK(cudaGetLastError());
    }
    return AGB_OK;
}

agb_status run_iter32(agb_solver s, int iter)
{
    agb_op op = s->op;
    const bool fc = iter < s->p.max_fmg_iter;
    if (s->p.use_graph) {
        if (s->g32 && s->g32_fcycle != (int)fc) {
            cudaGraphExecDestroy(s->g32);
            s->g32 = nullptr;
        }
        if (!s->g32) {
            const long long k0 = launch_counter();
            TRY(capture(op, &s->g32, [&] { iter32_body(s, fc ? 0 : s->p.max_fmg_iter); }));
            s->g32_kernels = launch_counter() - k0;
            launch_counter() = k0;
        }
        s->g32_fcycle = (int)fc;
        CK(cudaGraphLaunch(s->g32, op->st));
        s->replayed += s->g32_kernels;
    } else {
        iter32_body(s, iter);
        CK(cudaGetLastError());
    }
    return AGB_OK;
}

agb_status residual64(agb_solver s, double* norm)
{
    agb_op op = s->op;
    Engine<double> E{op, s->p};
    Level& v0 = op->lev[0];
    CK(cudaMemsetAsync(op->d_slots, 0, sizeof(double), op->st));
    E.fine_residual(s->x64, s->b64, v0.res64, op->d_slots);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(op->h_slots, op->d_slots, sizeof(double), cudaMemcpyDeviceToHost, op->st));
    double v;
    TRY(sync_read(op, &v, 1));
    *norm = op->h_slots[0];
    return AGB_OK;
}

agb_status norm64(agb_op op, const LevelDesc& L, const double* x, double* norm)
{
    CK(cudaMemsetAsync(op->d_slots + 2, 0, sizeof(double), op->st));
    launch_norm_inf<double>(op->st, L, 3, x, op->d_slots + 2);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(op->h_slots + 2, op->d_slots + 2, sizeof(double), cudaMemcpyDeviceToHost, op->st));
    CK(cudaStreamSynchronize(op->st));
    *norm = op->h_slots[2];
    return AGB_OK;
}


// The solve's first residual.  With a zero initial guess (a fresh solve,
// Newton's correction) r = b: A 0 = 0 holds exactly in every row (interior,
// displacement, traction and Neumann rows alike), so the FP64 operator
// application is skipped; b is already projected on a fully periodic box.
agb_status initial_residual(agb_solver s, double* res0)
{
    agb_op op = s->op;
    Level& v0 = op->lev[0];
    double xn;
    TRY(norm64(op, v0.L, s->x64, &xn));
    if (xn != 0) return residual64(s, res0);
    CK(cudaMemcpyAsync(v0.res64, s->b64, sizeof(double) * 3 * (size_t)v0.L.S, cudaMemcpyDeviceToDevice, op->st));
    return norm64(op, v0.L, v0.res64, res0);
}

// MLMG::solve restated on the resident (x64, b64); FP64 throughout.
agb_status solve_plain(agb_solver s, double tol_rel, double tol_abs, agb_solve_report* rep)
{
    agb_op op = s->op;
    double res0, bnorm;
    TRY(initial_residual(s, &res0));
    TRY(norm64(op, op->lev[0].L, s->b64, &bnorm));
    const double max_norm = bnorm >= res0 ? bnorm : res0;
    const double target = std::max(tol_abs, std::max(tol_rel, 1e-16) * max_norm);
    rep->res0 = res0;
    rep->rhs_norm = bnorm;
    rep->iterations = 0;
    double norm = res0;
    agb_status st = AGB_MAXITER;
    if (std::isnan(res0)) st = AGB_NAN;
    else if (res0 <= target) st = AGB_OK;
    else {
        for (int it = 0; it < s->p.max_iter; it++) {
            TRY(run_iter64(s, it));
            CK(cudaStreamSynchronize(op->st));
            norm = op->h_slots[0];
            rep->iterations = it + 1;
            if (s->p.verbose) fprintf(stderr, "agb MLMG iter %d resid %.6e rel %.6e\n", it + 1, norm, norm / max_norm);
            if (std::isnan(norm)) { st = AGB_NAN; break; }
            if (norm <= target) { st = AGB_OK; break; }
            if (s->p.fixed_iter > 0 && it + 1 >= s->p.fixed_iter) { st = AGB_OK; break; }
        }
    }
    rep->res_final = norm;
    return st;
}

// The preconditioner of the inner GCR: one FP32 cycle (F-cycle unless
// max_fmg_iter is 0) on the inner residual, leaving its result in cor32(0).
void precond32_body(agb_solver s)
{
    agb_op op = s->op;
    Engine<float> E{op, s->p};
    Level& v0 = op->lev[0];
    cudaMemcpyAsync(v0.res32, s->kr, sizeof(float) * 3 * (size_t)v0.L.S, cudaMemcpyDeviceToDevice, op->st);
    E.cycle(0);
}

agb_status run_precond32(agb_solver s)
{
    agb_op op = s->op;
    if (!s->p.use_graph) {
        precond32_body(s);
        CK(cudaGetLastError());
        return AGB_OK;
    }
    if (!s->gpre) {
        const long long k0 = launch_counter();
        TRY(capture(op, &s->gpre, [&] { precond32_body(s); }));
        s->gpre_kernels = launch_counter() - k0;
        launch_counter() = k0;
    }
    CK(cudaGraphLaunch(s->gpre, op->st));
    s->replayed += s->gpre_kernels;
    return AGB_OK;
}

// Inner solve A c = f (f = rhs32, c = sol32 zeroed by the caller) by flexible
// GCR with up to params.krylov stored directions (restarted when full): each
// iteration adds the direction z = M r, M one FP32 cycle, with w = A z
// orthogonalised against the stored w's (classical Gram-Schmidt) in the
// inner product <a, b> = sum a b / diag^2, and minimises the residual over
// it.  Every iteration lowers the weighted residual norm, whatever the
// orthogonality of the stored directions; the weights put displacement,
// traction and interior rows on one scale.  On a fully periodic box w is
// projected to zero mean like every residual.  Stops when max |r| <=
// inner_tol (f has max norm 1), when it stalls, or after inner_max_iter
// iterations (each one cycle).
agb_status inner_gcr32(agb_solver s, double inner_tol, double* inorm_out, int* cycles)
{
    agb_op op = s->op;
    Level& v0 = op->lev[0];
    const LevelDesc& L = v0.L;
    const int m = std::max(1, std::min(s->p.krylov, GCR_MAX));
    const long long n = 3 * L.S;
    const size_t bytes = sizeof(float) * (size_t)n;
    while ((int)s->kZ.size() < m) {
        float *z = nullptr, *w = nullptr;
        TRY(op->alloc(&z, (size_t)n));
        TRY(op->alloc(&w, (size_t)n));
        s->kZ.push_back(z);
        s->kW.push_back(w);
    }
    if (!s->kr) {
        TRY(op->alloc(&s->kr, (size_t)n));
        TRY(op->alloc(&s->kdots, GCR_MAX + 4));
    }
    cudaStream_t st = op->st;
    const bool sing = L.singular();
    CK(cudaMemcpyAsync(s->kr, s->rhs32, bytes, cudaMemcpyDeviceToDevice, st));
    double inorm = 1.0, prev = 1.0;
    int k = 0, slow = 0;
    for (int it = 0; it < s->p.inner_max_iter; it++) {
        if (k == m) k = 0;   // restart
        TRY(run_precond32(s));
        float* z = s->kZ[k];
        float* w = s->kW[k];
        CK(cudaMemcpyAsync(z, v0.cor32, bytes, cudaMemcpyDeviceToDevice, st));
        launch_stencil<float>(st, op->sym, MODE_APPLY, L, op->bc, op->uniform, v0.ddw32, z, nullptr, nullptr, w, 0.0f,
                              nullptr);
        if (sing) launch_remove_mean<float>(st, L, w, op->d_slots + 11);
        CK(cudaMemsetAsync(s->kdots, 0, sizeof(double) * (GCR_MAX + 2), st));
        if (k > 0) {
            GcrVecs W, Z;
            for (int i = 0; i < k; i++) {
                W.v[i] = s->kW[i];
                Z.v[i] = s->kZ[i];
            }
            launch_multidot_w(st, n, k, w, W, v0.dinv32, s->kdots);
            launch_gcr_orth(st, n, k, s->kdots, W, Z, w, z);
        }
        GcrVecs P;
        P.v[0] = w;
        P.v[1] = s->kr;
        launch_multidot_w(st, n, 2, w, P, v0.dinv32, s->kdots + GCR_MAX);
        CK(cudaMemsetAsync(op->d_slots + 1, 0, sizeof(double), st));
        launch_gcr_step(st, n, s->kdots + GCR_MAX, w, z, s->sol32, s->kr, op->d_slots + 1);
        CK(cudaMemcpyAsync(op->h_slots + 1, op->d_slots + 1, sizeof(double), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        inorm = slot_as_float(op->h_slots, 1);
        k++;
        (*cycles)++;
        if (s->p.verbose) fprintf(stderr, "agb mixed GCR inner %d resid32 %.3e\n", it + 1, inorm);
        if (std::isnan(inorm)) break;
        if (inorm <= inner_tol) break;
        if (s->net && s->learned_on) {
            // the learned direction on the residual the cycle left, kept only
            // if it removes at least learned_min_gain of the weighted residual
            // norm squared (after Gram-Schmidt against the stored directions)
            if (k == m) k = 0;
            float* zl = s->kZ[k];
            float* wl = s->kW[k];
            TRY(learned_direction(s->net, st, op->sym, L, s->kr, v0.ddw32, zl));
            launch_stencil<float>(st, op->sym, MODE_APPLY, L, op->bc, op->uniform, v0.ddw32, zl, nullptr, nullptr, wl,
                                  0.0f, nullptr);
            CK(cudaMemsetAsync(s->kdots, 0, sizeof(double) * (GCR_MAX + 4), st));
            if (k > 0) {
                GcrVecs W, Z;
                for (int i = 0; i < k; i++) {
                    W.v[i] = s->kW[i];
                    Z.v[i] = s->kZ[i];
                }
                launch_multidot_w(st, n, k, wl, W, v0.dinv32, s->kdots);
                launch_gcr_orth(st, n, k, s->kdots, W, Z, wl, zl);
            }
            GcrVecs P;
            P.v[0] = wl;
            P.v[1] = s->kr;
            launch_multidot_w(st, n, 2, wl, P, v0.dinv32, s->kdots + GCR_MAX);
            GcrVecs R;
            R.v[0] = s->kr;
            launch_multidot_w(st, n, 1, s->kr, R, v0.dinv32, s->kdots + GCR_MAX + 2);
            CK(cudaMemcpyAsync(op->h_slots + 4, s->kdots + GCR_MAX, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            const double ww = op->h_slots[4], wr = op->h_slots[5], rr = op->h_slots[6];
            const double gain = (ww > 0 && rr > 0) ? wr * wr / (ww * rr) : 0.0;
            s->learned_tried++;
            if (std::isfinite(gain) && gain >= s->learned_min_gain) {
                CK(cudaMemsetAsync(op->d_slots + 1, 0, sizeof(double), st));
                launch_gcr_step(st, n, s->kdots + GCR_MAX, wl, zl, s->sol32, s->kr, op->d_slots + 1);
                CK(cudaMemcpyAsync(op->h_slots + 1, op->d_slots + 1, sizeof(double), cudaMemcpyDeviceToHost, st));
                CK(cudaStreamSynchronize(st));
                inorm = slot_as_float(op->h_slots, 1);
                k++;
                s->learned_kept++;
                s->learned_fails = 0;
                if (s->p.verbose) fprintf(stderr, "agb learned direction kept: gain %.3e resid32 %.3e\n", gain, inorm);
                if (std::isnan(inorm)) break;
                if (inorm <= inner_tol) break;
            } else {
                if (++s->learned_fails >= s->learned_max_fail) s->learned_on = false;
                if (s->p.verbose) fprintf(stderr, "agb learned direction rejected: gain %.3e\n", gain);
            }
        }
        slow = (inorm > 0.9 * prev) ? slow + 1 : 0;
        if (slow >= 3) break;   // FP32 floor reached
        prev = inorm;
    }
    *inorm_out = inorm;
    return AGB_OK;
}

// FP32 cycles inside FP64 iterative refinement.
agb_status solve_mixed(agb_solver s, double tol_rel, double tol_abs, agb_solve_report* rep)
{
    agb_op op = s->op;
    TRY(ensure_f32(op));
    s->learned_on = s->net != nullptr && s->p.krylov > 0 && learned_level_ok(op->lev[0].L);
    s->learned_tried = s->learned_kept = s->learned_fails = 0;
    Level& v0 = op->lev[0];
    double res0, bnorm;
    TRY(initial_residual(s, &res0));
    TRY(norm64(op, v0.L, s->b64, &bnorm));
    const double max_norm = bnorm >= res0 ? bnorm : res0;
    const double target = std::max(tol_abs, std::max(tol_rel, 1e-16) * max_norm);
    rep->res0 = res0;
    rep->rhs_norm = bnorm;
    rep->iterations = 0;
    rep->refinements = 0;
    double norm = res0;
    if (std::isnan(res0)) { rep->res_final = res0; return AGB_NAN; }
    if (res0 <= target) { rep->res_final = res0; return AGB_OK; }
    agb_status st = AGB_MAXITER;
    int total_cycles = 0, no_progress = 0;
    const size_t bytes32 = sizeof(float) * 3 * (size_t)v0.L.S;
    for (int outer = 0; outer < s->p.max_refine; outer++) {
        const double scale = 1.0 / norm;
        // inner problem: A c = r / ||r||, FP32, c0 = 0
        launch_convert<float, double>(op->st, v0.L, 3, v0.res64, s->rhs32, scale);
        CK(cudaMemsetAsync(s->sol32, 0, bytes32, op->st));
        CK(cudaMemcpyAsync(v0.res32, s->rhs32, bytes32, cudaMemcpyDeviceToDevice, op->st));
        const double inner_tol = std::max(s->p.inner_tol_rel, 0.3 * target / norm);
        double inorm = 1.0, prev = 1.0;
        int slow = 0;
        if (s->p.krylov > 0) TRY(inner_gcr32(s, inner_tol, &inorm, &total_cycles));
        for (int it = 0; s->p.krylov <= 0 && it < s->p.inner_max_iter; it++) {
            TRY(run_iter32(s, it));
            CK(cudaStreamSynchronize(op->st));
            inorm = slot_as_float(op->h_slots, 1);
            total_cycles++;
            if (s->p.verbose) fprintf(stderr, "agb mixed outer %d inner %d resid32 %.3e\n", outer, it + 1, inorm);
            if (std::isnan(inorm)) break;
            if (inorm <= inner_tol) break;
            slow = (inorm > 0.9 * prev) ? slow + 1 : 0;
            if (slow >= 3) break;   // FP32 floor reached
            prev = inorm;
        }
        if (std::isnan(inorm)) { st = AGB_NAN; break; }
        launch_axpy_mixed(op->st, v0.L, 3, s->x64, s->sol32, 1.0 / scale);
        CK(cudaGetLastError());
        const double old = norm;
        TRY(residual64(s, &norm));
        rep->refinements++;
        if (s->p.verbose)
            fprintf(stderr, "agb mixed outer %d resid64 %.6e rel %.6e\n", outer, norm, norm / max_norm);
        if (std::isnan(norm)) { st = AGB_NAN; break; }
        if (norm <= target) { st = AGB_OK; break; }
        no_progress = (norm > 0.5 * old) ? no_progress + 1 : 0;
        if (no_progress >= 1) s->learned_on = false;   // the FP64 residual decides: plain cycles from here
        if (no_progress >= 2) { st = AGB_STALL; break; }
    }
    rep->iterations = total_cycles;
    rep->res_final = norm;
    return st;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char* agb_last_error(void) { return g_err.c_str(); }
const char* agb_version(void) { return "alamo_gb300 0.1 (sm_103a)"; }

void agb_default_params(agb_solver_params* p)
{
    p->max_iter = 200;
    p->fixed_iter = -1;
    p->pre_smooth = 2;
    p->post_smooth = 2;
    p->final_smooth = 8;
    p->bottom_smooth = 0;
    p->max_fmg_iter = 100000000;
    p->bottom_max_iter = 200;
    p->bottom_tol_rel = 1e-4;
    p->bottom_tol_abs = -1.0;
    p->omega = -1.0;   // keep the operator's (2/3 unless agb_op_set_omega)
    p->max_coarsening_level = 30;
    p->verbose = 0;
    p->precision = AGB_PREC_F64;
    p->inner_tol_rel = 1e-4;
    p->inner_max_iter = 60;
    p->max_refine = 20;
    p->use_graph = 1;
    p->krylov = 0;
}

agb_status agb_op_create(const int n_cells[3], const double dx[3], const int periodic[3], int sym,
                         int max_coarsening_level, agb_op* out)
{
    if (!out || !n_cells || !dx) return fail(AGB_BADARG, "null argument");
    *out = nullptr;
    if (sym != AGB_ISO && sym != AGB_MAJORMINOR) return fail(AGB_BADARG, "sym must be AGB_ISO or AGB_MAJORMINOR");
    for (int d = 0; d < 3; d++) {
        if (n_cells[d] < 2) return fail(AGB_BADARG, "n_cells[%d]=%d must be >= 2", d, n_cells[d]);
        if (!(dx[d] > 0)) return fail(AGB_BADARG, "dx[%d] must be positive", d);
    }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(AGB_CUDA, "no usable CUDA device (%s)", cudaGetErrorString(e));
    }
    agb_op op = new (std::nothrow) agb_op_s();
    if (!op) return fail(AGB_NOMEM, "host allocation failed");
    op->sym = sym;
    op->nc = sym == AGB_ISO ? 2 : 21;
    for (int d = 0; d < 3; d++) {
        op->n[d] = n_cells[d];
        op->per[d] = periodic ? (periodic[d] ? 1 : 0) : 0;
        op->dx[d] = dx[d];
    }
    memset(&op->bc, 0, sizeof(op->bc));
    auto bail = [&](agb_status s) {
        agb_op_destroy(op);
        return s;
    };
    if (cudaStreamCreateWithFlags(&op->st, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(AGB_CUDA, "cudaStreamCreate failed"));
    cudaEventCreate(&op->e0);
    cudaEventCreate(&op->e1);
    if (!g_attr_done) {
        init_kernel_attributes();
        init_bottom_attributes();
        init_tma_attributes();
        g_attr_done = true;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&op->pageable_ok, cudaDevAttrPageableMemoryAccess, dev);
    const int nl = num_levels(n_cells, max_coarsening_level < 0 ? 30 : max_coarsening_level);
    int n[3] = {n_cells[0], n_cells[1], n_cells[2]};
    double h[3] = {dx[0], dx[1], dx[2]};
    for (int l = 0; l < nl; l++) {
        Level lv;
        lv.L = make_level(n, op->per, h);
        op->lev.push_back(lv);
        for (int d = 0; d < 3; d++) {
            n[d] /= 2;
            h[d] *= 2.0;
        }
    }
    for (auto& lv : op->lev) {
        const size_t n3 = 3 * (size_t)lv.L.S;
        agb_status s;
        if ((s = op->alloc(&lv.ddw64, op->nc * (size_t)lv.L.S)) != AGB_OK) return bail(s);
        if ((s = op->alloc(&lv.diag64, n3)) != AGB_OK) return bail(s);
        if ((s = op->alloc(&lv.dinv64, n3)) != AGB_OK) return bail(s);
        if ((s = op->alloc(&lv.cor64, n3)) != AGB_OK) return bail(s);
        if ((s = op->alloc(&lv.res64, n3)) != AGB_OK) return bail(s);
        if ((s = op->alloc(&lv.rescor64, n3)) != AGB_OK) return bail(s);
        if ((s = op->alloc(&lv.hold64, n3)) != AGB_OK) return bail(s);
        if ((s = op->alloc(&lv.tmp64, n3)) != AGB_OK) return bail(s);
    }
    agb_status s;
    if ((s = op->alloc(&op->d_slots, 16)) != AGB_OK) return bail(s);
    if ((s = op->alloc(&op->bottom_work, 8 * 3 * (size_t)op->lev.back().L.S)) != AGB_OK) return bail(s);
    if ((s = op->alloc(&op->d_ret, 4)) != AGB_OK) return bail(s);
    if (bottom_dense_fits(op->lev.back().L) && use_dense_bottom()) {
        if ((s = op->alloc(&op->bottom_A, bottom_dense_bytes(op->lev.back().L) / sizeof(double))) != AGB_OK)
            return bail(s);
        if (use_exact_bottom()) {
            if ((s = op->alloc(&op->bottom_inv32, bottom_dense_bytes(op->lev.back().L) / sizeof(double))) != AGB_OK)
                return bail(s);
            if ((s = op->alloc(&op->bottom_inv_ok, 1)) != AGB_OK) return bail(s);
        }
    }
    op->stage_bytes = 64u << 20;
    if ((s = op->alloc(&op->stage, op->stage_bytes)) != AGB_OK) return bail(s);
    if (cudaMallocHost(&op->h_slots, 16 * sizeof(double)) != cudaSuccess)
        return bail(fail(AGB_NOMEM, "cudaMallocHost failed"));
    if (cudaStreamSynchronize(op->st) != cudaSuccess) return bail(fail(AGB_CUDA, "stream sync failed"));
    *out = op;
    return AGB_OK;
}

agb_status agb_op_destroy(agb_op op)
{
    if (!op) return AGB_OK;
    if (op->st) cudaStreamSynchronize(op->st);
    for (void* p : op->allocs) cudaFree(p);
    if (op->dma) cudaFree(op->dma);
    if (op->h_slots) cudaFreeHost(op->h_slots);
    if (op->e0) cudaEventDestroy(op->e0);
    if (op->e1) cudaEventDestroy(op->e1);
    if (op->st) cudaStreamDestroy(op->st);
    delete op;
    return AGB_OK;
}

agb_status agb_op_set_bc(agb_op op, const agb_bc* bc)
{
    if (!op || !bc) return fail(AGB_BADARG, "null argument");
    for (int f = 0; f < AGB_NFACES; f++)
        for (int c = 0; c < 3; c++) {
            const int t = bc->type[f][c];
            if (t < AGB_BC_DISP || t > AGB_BC_NONE) return fail(AGB_BADARG, "bad BC type %d at face %d comp %d", t, f, c);
            op->bc.type[f][c] = (int8_t)t;
            op->bc.val[f][c] = bc->val[f][c];
        }
    op->bc_set = true;
    op->prepared = false;
    return AGB_OK;
}

agb_status agb_op_set_model(agb_op op, const double* ddw, int layout, int mem)
{
    if (!op || !ddw) return fail(AGB_BADARG, "null argument");
    if (layout != AGB_LAYOUT_AOS && layout != AGB_LAYOUT_SOA) return fail(AGB_BADARG, "bad layout");
    TRY(upload<double, double>(op, op->lev[0].L, op->nc, layout == AGB_LAYOUT_AOS, ddw, mem, op->lev[0].ddw64));
    CK(cudaStreamSynchronize(op->st));
    op->model_set = true;
    op->prepared = false;
    op->f32_ready = false;
    return AGB_OK;
}

agb_status agb_op_set_uniform(agb_op op, int uniform)
{
    if (!op) return fail(AGB_BADARG, "null operator");
    op->uniform = uniform != 0;
    return AGB_OK;
}

agb_status agb_op_set_omega(agb_op op, double omega)
{
    if (!op) return fail(AGB_BADARG, "null operator");
    if (!(omega > 0 && omega < 2)) return fail(AGB_BADARG, "omega must be in (0,2)");
    op->omega = omega;
    return AGB_OK;
}

agb_status agb_op_num_levels(agb_op op, int* nlevels)
{
    if (!op || !nlevels) return fail(AGB_BADARG, "null argument");
    *nlevels = (int)op->lev.size();
    return AGB_OK;
}

agb_status agb_op_level_cells(agb_op op, int level, int n_cells[3])
{
    TRY(check_level(op, level));
    for (int d = 0; d < 3; d++) n_cells[d] = op->lev[level].L.n[d];
    return AGB_OK;
}

agb_status agb_op_prepare(agb_op op)
{
    if (!op) return fail(AGB_BADARG, "null operator");
    TRY(prepare(op));
    CK(cudaStreamSynchronize(op->st));
    return AGB_OK;
}

agb_status agb_op_get_model(agb_op op, int level, double* ddw, int layout, int mem)
{
    TRY(check_level(op, level));
    TRY(prepare(op));
    Level& v = op->lev[level];
    TRY((download<double, double>(op, v.L, op->nc, layout == AGB_LAYOUT_AOS, v.ddw64, ddw, mem)));
    CK(cudaStreamSynchronize(op->st));
    return AGB_OK;
}

agb_status agb_op_fapply(agb_op op, int level, double* f, const double* u, int mem)
{
    TRY(check_level(op, level));
    TRY(prepare(op));
    Level& v = op->lev[level];
    TRY((upload<double, double>(op, v.L, 3, false, u, mem, v.hold64)));
    launch_stencil<double>(op->st, op->sym, MODE_APPLY, v.L, op->bc, op->uniform, v.ddw64, v.hold64, nullptr, nullptr,
                           v.tmp64, 0.0, nullptr);
    CK(cudaGetLastError());
    TRY((download<double, double>(op, v.L, 3, false, v.tmp64, f, mem)));
    CK(cudaStreamSynchronize(op->st));
    return AGB_OK;
}

agb_status agb_op_fapply_f32(agb_op op, int level, float* f, const float* u, int mem)
{
    TRY(check_level(op, level));
    TRY(prepare(op));
    TRY(ensure_f32(op));
    Level& v = op->lev[level];
    TRY((upload<float, float>(op, v.L, 3, false, u, mem, v.hold32)));
    launch_stencil<float>(op->st, op->sym, MODE_APPLY, v.L, op->bc, op->uniform, v.ddw32, v.hold32, nullptr, nullptr,
                          v.tmp32, 0.0f, nullptr);
    CK(cudaGetLastError());
    TRY((download<float, float>(op, v.L, 3, false, v.tmp32, f, mem)));
    CK(cudaStreamSynchronize(op->st));
    return AGB_OK;
}

agb_status agb_op_diagonal(agb_op op, int level, double* diag, int mem)
{
    TRY(check_level(op, level));
    TRY(prepare(op));
    Level& v = op->lev[level];
    TRY((download<double, double>(op, v.L, 3, false, v.diag64, diag, mem)));
    CK(cudaStreamSynchronize(op->st));
    return AGB_OK;
}

agb_status agb_op_fsmooth(agb_op op, int level, double* x, const double* b, int mem)
{
    TRY(check_level(op, level));
    TRY(prepare(op));
    Level& v = op->lev[level];
    TRY((upload<double, double>(op, v.L, 3, false, x, mem, v.hold64)));
    TRY((upload<double, double>(op, v.L, 3, false, b, mem, v.rescor64)));
    agb_solver_params p;
    agb_default_params(&p);
    Engine<double> E{op, p};
    E.smooth(level, v.hold64, v.rescor64, 1);
    CK(cudaGetLastError());
    TRY((download<double, double>(op, v.L, 3, false, v.hold64, x, mem)));
    CK(cudaStreamSynchronize(op->st));
    return AGB_OK;
}

agb_status agb_op_fsmooth_f32(agb_op op, int level, float* x, const float* b, int mem)
{
    TRY(check_level(op, level));
    TRY(prepare(op));
    TRY(ensure_f32(op));
    Level& v = op->lev[level];
    TRY((upload<float, float>(op, v.L, 3, false, x, mem, v.hold32)));
    TRY((upload<float, float>(op, v.L, 3, false, b, mem, v.rescor32)));
    agb_solver_params p;
    agb_default_params(&p);
    Engine<float> E{op, p};
    E.smooth(level, v.hold32, v.rescor32, 1);
    CK(cudaGetLastError());
    TRY((download<float, float>(op, v.L, 3, false, v.hold32, x, mem)));
    CK(cudaStreamSynchronize(op->st));
    return AGB_OK;
}

agb_status agb_op_residual(agb_op op, int level, double* r, const double* x, const double* b, int mem)
{
    TRY(check_level(op, level));
    TRY(prepare(op));
    Level& v = op->lev[level];
    TRY((upload<double, double>(op, v.L, 3, false, x, mem, v.hold64)));
    TRY((upload<double, double>(op, v.L, 3, false, b, mem, v.rescor64)));
    launch_stencil<double>(op->st, op->sym, MODE_RESID, v.L, op->bc, op->uniform, v.ddw64, v.hold64, v.rescor64,
                           nullptr, v.tmp64, 0.0, nullptr);
    CK(cudaGetLastError());
    TRY((download<double, double>(op, v.L, 3, false, v.tmp64, r, mem)));
    CK(cudaStreamSynchronize(op->st));
    return AGB_OK;
}

agb_status agb_op_restriction(agb_op op, int crse_level, double* crse, const double* fine, int mem)
{
    TRY(check_level(op, crse_level));
    if (crse_level < 1) return fail(AGB_BADARG, "crse_level must be >= 1");
    Level& f = op->lev[crse_level - 1];
    Level& c = op->lev[crse_level];
    TRY((upload<double, double>(op, f.L, 3, false, fine, mem, f.hold64)));
    launch_restriction<double>(op->st, f.L, c.L, f.hold64, c.tmp64, 3);
    CK(cudaGetLastError());
    TRY((download<double, double>(op, c.L, 3, false, c.tmp64, crse, mem)));
    CK(cudaStreamSynchronize(op->st));
    return AGB_OK;
}

agb_status agb_op_interpolation(agb_op op, int fine_level, double* fine, const double* crse, int mem)
{
    TRY(check_level(op, fine_level));
    if (fine_level + 1 >= (int)op->lev.size()) return fail(AGB_BADARG, "fine_level has no coarser level");
    Level& f = op->lev[fine_level];
    Level& c = op->lev[fine_level + 1];
    TRY((upload<double, double>(op, f.L, 3, false, fine, mem, f.hold64)));
    TRY((upload<double, double>(op, c.L, 3, false, crse, mem, c.hold64)));
    launch_interpolation<double>(op->st, f.L, c.L, f.hold64, c.hold64, false);
    CK(cudaGetLastError());
    TRY((download<double, double>(op, f.L, 3, false, f.hold64, fine, mem)));
    CK(cudaStreamSynchronize(op->st));
    return AGB_OK;
}

agb_status agb_solver_create(agb_op op, const agb_solver_params* params, agb_solver* out)
{
    if (!op || !out) return fail(AGB_BADARG, "null argument");
    *out = nullptr;
    agb_solver s = new (std::nothrow) agb_solver_s();
    if (!s) return fail(AGB_NOMEM, "host allocation failed");
    s->op = op;
    if (params) s->p = *params;
    else agb_default_params(&s->p);
    if (s->p.precision != AGB_PREC_F64 && s->p.precision != AGB_PREC_MIXED) {
        delete s;
        return fail(AGB_BADARG, "bad precision");
    }
    if (s->p.krylov < 0 || s->p.krylov > GCR_MAX) {
        delete s;
        return fail(AGB_BADARG, "krylov must be in 0..%d", GCR_MAX);
    }
    if (s->p.omega > 0) op->omega = s->p.omega;   // Linear::PrepareMLMG -> SetOmega
    const size_t n3 = 3 * (size_t)op->lev[0].L.S;
    agb_status st;
    if ((st = op->alloc(&s->x64, n3)) != AGB_OK || (st = op->alloc(&s->b64, n3)) != AGB_OK) {
        delete s;
        return st;
    }
    if (s->p.precision == AGB_PREC_MIXED) {
        if ((st = op->alloc(&s->rhs32, n3)) != AGB_OK || (st = op->alloc(&s->sol32, n3)) != AGB_OK) {
            delete s;
            return st;
        }
    }
    *out = s;
    return AGB_OK;
}

agb_status agb_solver_destroy(agb_solver s)
{
    if (!s) return AGB_OK;
    if (s->g64) cudaGraphExecDestroy(s->g64);
    if (s->g32) cudaGraphExecDestroy(s->g32);
    if (s->gpre) cudaGraphExecDestroy(s->gpre);
    delete s;
    return AGB_OK;
}

static agb_status solve_resident(agb_solver s, double tol_rel, double tol_abs, agb_solve_report* rep)
{
    agb_op op = s->op;
    rep->nlevels = (int)op->lev.size();
    rep->refinements = 0;
    const LevelDesc& L0 = op->lev[0].L;
    // fully periodic box: solve with the zero-mean part of b (Engine::fine_residual)
    if (L0.singular()) launch_remove_mean<double>(op->st, L0, s->b64, op->d_slots + 8);
    const agb_status st =
        s->p.precision == AGB_PREC_MIXED ? solve_mixed(s, tol_rel, tol_abs, rep) : solve_plain(s, tol_rel, tol_abs, rep);
    // and return the displacement modulo rigid translation: zero mean
    if (L0.singular()) launch_remove_mean<double>(op->st, L0, s->x64, op->d_slots + 8);
    CK(cudaStreamSynchronize(op->st));
    if (tma_error_take()) return fail(AGB_CUDA, "a TMA plane copy of the stencil kernel did not complete in time");
    return st;
}

agb_status agb_solve(agb_solver s, double* sol, const double* rhs, double tol_rel, double tol_abs, int mem,
                     agb_solve_report* report)
{
    if (!s || !sol || !rhs) return fail(AGB_BADARG, "null argument");
    agb_op op = s->op;
    agb_solve_report rep;
    memset(&rep, 0, sizeof(rep));
    const long long k0 = launch_counter();
    s->replayed = 0;
    CK(cudaEventRecord(op->e0, op->st));
    TRY(prepare_for_solve(s));
    TRY((upload<double, double>(op, op->lev[0].L, 3, false, sol, mem, s->x64)));
    TRY((upload<double, double>(op, op->lev[0].L, 3, false, rhs, mem, s->b64)));
    agb_status st = solve_resident(s, tol_rel, tol_abs, &rep);
    if (st == AGB_CUDA || st == AGB_NOMEM || st == AGB_BADARG || st == AGB_STATE) return st;
    TRY((download<double, double>(op, op->lev[0].L, 3, false, s->x64, sol, mem)));
    CK(cudaEventRecord(op->e1, op->st));
    CK(cudaStreamSynchronize(op->st));
    float ms = 0;
    cudaEventElapsedTime(&ms, op->e0, op->e1);
    rep.solve_ms = ms;
    rep.status = st;
    rep.kernels = launch_counter() - k0 + s->replayed;
    if (report) *report = rep;
    if (st != AGB_OK) fail(st, "solve did not converge: status %d after %d iterations, |r| %.3e (target from |r0| %.3e)",
                           (int)st, rep.iterations, rep.res_final, rep.res0);
    return st;
}

// Flexible GCR with a V-cycle (+ learned correction) preconditioner; see agb.h.
agb_status agb_solver_set_learned(agb_solver s, agb_learned net, double min_gain, int max_fail)
{
    if (!s) return fail(AGB_BADARG, "null solver");
    if (net && !learned_level_ok(s->op->lev[0].L))
        return fail(AGB_BADARG, "the learned correction needs a box with no periodic direction and edges divisible by 4");
    if (!(min_gain >= 0 && min_gain < 1) || max_fail < 1) return fail(AGB_BADARG, "min_gain in [0,1), max_fail >= 1");
    s->net = net;
    s->learned_min_gain = min_gain;
    s->learned_max_fail = max_fail;
    return AGB_OK;
}

agb_status agb_solver_learned_stats(agb_solver s, int* tried, int* kept, int* active)
{
    if (!s || !tried || !kept || !active) return fail(AGB_BADARG, "null argument");
    *tried = s->learned_tried;
    *kept = s->learned_kept;
    *active = s->learned_on ? 1 : 0;
    return AGB_OK;
}

agb_status agb_unet_features(agb_op op, const double* r, int mem, void* feat, double* rms)
{
    TRY(check_level(op, 0));
    if (!r || !feat || !rms) return fail(AGB_BADARG, "null argument");
    Level& v = op->lev[0];
    if (!learned_level_ok(v.L))
        return fail(AGB_BADARG, "the learned correction needs a box with no periodic direction and edges divisible by 4");
    TRY(prepare(op));
    TRY(ensure_f32(op));
    TRY((upload<float, double>(op, v.L, 3, false, r, mem, v.hold32)));
    TRY(learned_features(op->st, op->sym, v.L, v.hold32, v.ddw32, feat, op->d_slots + 4));
    CK(cudaMemcpyAsync(op->h_slots + 4, op->d_slots + 4, sizeof(double), cudaMemcpyDeviceToHost, op->st));
    CK(cudaStreamSynchronize(op->st));
    *rms = std::sqrt(op->h_slots[4] / (3.0 * (double)v.L.count()));
    return AGB_OK;
}

agb_status agb_apply(agb_solver s, double* out, const double* in, int mem)
{
    if (!s) return fail(AGB_BADARG, "null solver");
    return agb_op_fapply(s->op, 0, out, in, mem);
}

agb_status agb_bc_init(agb_op op, double* rhs, int homogeneous, int mem)
{
    if (!op || !rhs) return fail(AGB_BADARG, "null argument");
    if (!op->bc_set) return fail(AGB_STATE, "SetBC must be called first");
    Level& v = op->lev[0];
    TRY((upload<double, double>(op, v.L, 3, false, rhs, mem, v.tmp64)));
    launch_bc_init(op->st, v.L, op->bc, v.tmp64, homogeneous);
    CK(cudaGetLastError());
    TRY((download<double, double>(op, v.L, 3, false, v.tmp64, rhs, mem)));
    CK(cudaStreamSynchronize(op->st));
    return AGB_OK;
}

// A finest-level work field kept by the operator across calls (allocated once).
static agb_status kept(agb_op op, double** slot, size_t count)
{
    if (!*slot) TRY(op->alloc(slot, count));
    return AGB_OK;
}

static agb_status load_F0(agb_op op, const double* F0, int mem, double** dF0)
{
    *dF0 = nullptr;
    if (!F0) return AGB_OK;
    Level& v = op->lev[0];
    TRY(kept(op, &op->nw_F0, 9 * (size_t)v.L.S));
    TRY((upload<double, double>(op, v.L, 9, true, F0, mem, op->nw_F0)));
    *dF0 = op->nw_F0;
    return AGB_OK;
}

static void release(agb_op op, void* p)
{
    if (!p) return;
    cudaStreamSynchronize(op->st);
    cudaFree(p);
    op->allocs.erase(std::remove(op->allocs.begin(), op->allocs.end(), p), op->allocs.end());
}

agb_status agb_newton_rhs(agb_op op, const double* F0, const double* u, const double* b, double* rhs, int mem)
{
    if (!op || !u || !b || !rhs) return fail(AGB_BADARG, "null argument");
    if (!op->model_set || !op->bc_set) return fail(AGB_STATE, "SetModel and SetBC must be called first");
    Level& v = op->lev[0];
    double *dF0 = nullptr, *dw = nullptr;
    TRY(load_F0(op, F0, mem, &dF0));
    agb_status st = kept(op, &op->nw_dw, 9 * (size_t)v.L.S);
    dw = op->nw_dw;
    if (st == AGB_OK) st = upload<double, double>(op, v.L, 3, false, u, mem, v.hold64);
    if (st == AGB_OK) st = upload<double, double>(op, v.L, 3, false, b, mem, v.rescor64);
    if (st == AGB_OK) {
        launch_newton_rhs(op->st, op->sym, v.L, op->bc, v.ddw64, dF0, v.hold64, v.rescor64, v.tmp64, dw);
        if (cudaGetLastError() != cudaSuccess) st = fail(AGB_CUDA, "newton rhs launch failed");
    }
    if (st == AGB_OK) st = download<double, double>(op, v.L, 3, false, v.tmp64, rhs, mem);
    if (st == AGB_OK && cudaStreamSynchronize(op->st) != cudaSuccess) st = fail(AGB_CUDA, "newton rhs failed");
    return st;
}

agb_status agb_newton_solve(agb_solver s, const double* F0, double* u, const double* b, double tol_rel,
                            double tol_abs, int mem, agb_solve_report* report)
{
    if (!s || !u || !b) return fail(AGB_BADARG, "null argument");
    agb_op op = s->op;
    Level& v = op->lev[0];
    double *dF0 = nullptr, *dw = nullptr, *u0 = nullptr;
    agb_solve_report rep;
    memset(&rep, 0, sizeof(rep));
    const long long k0 = launch_counter();
    s->replayed = 0;
    CK(cudaEventRecord(op->e0, op->st));
    TRY(prepare_for_solve(s));
    TRY(load_F0(op, F0, mem, &dF0));
    agb_status st = kept(op, &op->nw_dw, 9 * (size_t)v.L.S);
    if (st == AGB_OK) st = kept(op, &op->nw_u0, 3 * (size_t)v.L.S);
    dw = op->nw_dw;
    u0 = op->nw_u0;
    if (st == AGB_OK) st = upload<double, double>(op, v.L, 3, false, u, mem, u0);
    if (st == AGB_OK) st = upload<double, double>(op, v.L, 3, false, b, mem, v.rescor64);
    double unorm = 1.0;
    if (st == AGB_OK && !dF0) st = norm64(op, v.L, u0, &unorm);
    if (st == AGB_OK) {
        // Newton.H:323: rhs from the current u; Linear::solve for dsol from 0.
        // Without an eigenstrain and from u = 0, DW = C : grad 0 = 0 and every
        // row of div DW and of the BC rows is exactly 0: rhs = b.
        if (!dF0 && unorm == 0.0)
            cudaMemcpyAsync(s->b64, v.rescor64, sizeof(double) * 3 * (size_t)v.L.S, cudaMemcpyDeviceToDevice, op->st);
        else
            launch_newton_rhs(op->st, op->sym, v.L, op->bc, v.ddw64, dF0, u0, v.rescor64, s->b64, dw);
        cudaMemsetAsync(s->x64, 0, sizeof(double) * 3 * (size_t)v.L.S, op->st);
        if (cudaGetLastError() != cudaSuccess) st = fail(AGB_CUDA, "newton rhs launch failed");
    }
    agb_status sst = AGB_OK;
    if (st == AGB_OK) {
        sst = solve_resident(s, tol_rel, tol_abs, &rep);
        if (sst == AGB_CUDA || sst == AGB_NOMEM || sst == AGB_STATE || sst == AGB_BADARG) st = sst;
    }
    if (st == AGB_OK) {
        launch_axpy<double>(op->st, v.L, 3, u0, s->x64, 1.0);   // Newton.H:348-349
        st = download<double, double>(op, v.L, 3, false, u0, u, mem);
    }
    if (st == AGB_OK) {
        cudaEventRecord(op->e1, op->st);
        if (cudaStreamSynchronize(op->st) != cudaSuccess) st = fail(AGB_CUDA, "newton solve failed");
        float ms = 0;
        cudaEventElapsedTime(&ms, op->e0, op->e1);
        rep.solve_ms = ms;
    }
    rep.status = st == AGB_OK ? sst : st;
    rep.kernels = launch_counter() - k0 + s->replayed;
    if (report) *report = rep;
    return st == AGB_OK ? sst : st;
}

agb_status agb_stress(agb_op op, const double* F0, const double* u, double* sigma9, int mem)
{
    if (!op || !u || !sigma9) return fail(AGB_BADARG, "null argument");
    if (!op->model_set) return fail(AGB_STATE, "SetModel must be called first");
    Level& v = op->lev[0];
    double *dF0 = nullptr, *sg = nullptr;
    TRY(load_F0(op, F0, mem, &dF0));
    agb_status st = op->alloc(&sg, 9 * (size_t)v.L.S);
    if (st == AGB_OK) st = upload<double, double>(op, v.L, 3, false, u, mem, v.hold64);
    if (st == AGB_OK) {
        launch_stress(op->st, op->sym, v.L, v.ddw64, dF0, v.hold64, sg);
        st = download<double, double>(op, v.L, 9, true, sg, sigma9, mem);
    }
    if (st == AGB_OK && cudaStreamSynchronize(op->st) != cudaSuccess) st = fail(AGB_CUDA, "stress failed");
    release(op, sg);
    return st;
}

agb_status agb_strain_energy(agb_op op, const double* u, double* eps9, double* energy, int mem)
{
    if (!op || !u || (!eps9 && !energy)) return fail(AGB_BADARG, "null argument");
    if (!op->model_set) return fail(AGB_STATE, "SetModel must be called first");
    Level& v = op->lev[0];
    double *de = nullptr, *dw = nullptr;
    agb_status st = AGB_OK;
    if (eps9) st = op->alloc(&de, 9 * (size_t)v.L.S);
    if (st == AGB_OK && energy) st = op->alloc(&dw, (size_t)v.L.S);
    if (st == AGB_OK) st = upload<double, double>(op, v.L, 3, false, u, mem, v.hold64);
    if (st == AGB_OK) {
        launch_strain_energy(op->st, op->sym, v.L, v.ddw64, v.hold64, de, dw);
        if (cudaGetLastError() != cudaSuccess) st = fail(AGB_CUDA, "strain/energy launch failed");
    }
    if (st == AGB_OK && eps9) st = download<double, double>(op, v.L, 9, true, de, eps9, mem);
    if (st == AGB_OK && energy) st = download<double, double>(op, v.L, 1, false, dw, energy, mem);
    if (st == AGB_OK && cudaStreamSynchronize(op->st) != cudaSuccess) st = fail(AGB_CUDA, "strain/energy failed");
    if (de) release(op, de);
    if (dw) release(op, dw);
    return st;
}

agb_status agb_traction_xhi(agb_op op, const double* F0, const double* u, double trac[3], int mem)
{
    if (!op || !u || !trac) return fail(AGB_BADARG, "null argument");
    if (!op->model_set) return fail(AGB_STATE, "SetModel must be called first");
    Level& v = op->lev[0];
    double *dF0 = nullptr, *sg = nullptr;
    TRY(load_F0(op, F0, mem, &dF0));
    agb_status st = op->alloc(&sg, 9 * (size_t)v.L.S);
    if (st == AGB_OK) st = upload<double, double>(op, v.L, 3, false, u, mem, v.hold64);
    if (st == AGB_OK) {
        launch_stress(op->st, op->sym, v.L, v.ddw64, dF0, v.hold64, sg);
        launch_traction_xhi(op->st, v.L, sg, op->d_slots + 4);
        if (cudaMemcpyAsync(op->h_slots + 4, op->d_slots + 4, 3 * sizeof(double), cudaMemcpyDeviceToHost, op->st) !=
                cudaSuccess ||
            cudaStreamSynchronize(op->st) != cudaSuccess)
            st = fail(AGB_CUDA, "traction failed");
        else
            for (int r = 0; r < 3; r++) trac[r] = op->h_slots[4 + r];
    }
    release(op, sg);
    return st;
}

agb_status agb_op_time_sweep(agb_op op, int level, int precision, int mode, int reps, double* ms_per_launch)
{
    TRY(check_level(op, level));
    if (!ms_per_launch || reps < 1 || mode < 0 || mode > 2) return fail(AGB_BADARG, "bad argument");
    TRY(prepare(op));
    Level& v = op->lev[level];
    if (precision == AGB_PREC_MIXED) TRY(ensure_f32(op));
    auto one = [&]() {
        if (precision == AGB_PREC_MIXED)
            launch_stencil<float>(op->st, op->sym, mode, v.L, op->bc, op->uniform, v.ddw32, v.cor32, v.res32, v.dinv32,
                                  v.tmp32, (float)op->omega, mode == MODE_RESID ? (void*)(op->d_slots + 3) : nullptr);
        else
            launch_stencil<double>(op->st, op->sym, mode, v.L, op->bc, op->uniform, v.ddw64, v.cor64, v.res64, v.dinv64,
                                   v.tmp64, op->omega, mode == MODE_RESID ? (void*)(op->d_slots + 3) : nullptr);
    };
    one();
    CK(cudaGetLastError());
    CK(cudaEventRecord(op->e0, op->st));
    for (int r = 0; r < reps; r++) one();
    CK(cudaEventRecord(op->e1, op->st));
    CK(cudaEventSynchronize(op->e1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, op->e0, op->e1));
    *ms_per_launch = ms / reps;
    if (tma_error_take()) return fail(AGB_CUDA, "a TMA plane copy of the stencil kernel did not complete in time");
    return AGB_OK;
}

agb_status agb_host_alloc(size_t bytes, void** p)
{
    if (!p) return fail(AGB_BADARG, "null argument");
    CK(cudaMallocHost(p, bytes));
    return AGB_OK;
}

agb_status agb_host_free(void* p)
{
    CK(cudaFreeHost(p));
    return AGB_OK;
}

}  // extern "C"
