// kernels_peak.cu -- measured FP64 FMA throughput of the device, the
// denominator of the FP64 stencils' roofline (their bound is the FP64 pipe,
// not HBM).  The kernel runs 8 independent fused-multiply-add chains per
// thread on every SM; the host times it with CUDA events on its own stream.

#include "../../include/agb.h"
#include "agb_internal.h"

namespace {

constexpr int CHAINS = 8;
constexpr int UNROLL = 16;

__global__ void __launch_bounds__(256) k_fp64_fma(double* sink, int iters, double m, double a)
{
    double x[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; c++) x[c] = 1e-3 * (threadIdx.x + 1) + c;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int r = 0; r < UNROLL; r++) {
#pragma unroll
            for (int c = 0; c < CHAINS; c++) x[c] = fma(x[c], m, a);
        }
    }
    double s = 0;
#pragma unroll
    for (int c = 0; c < CHAINS; c++) s += x[c];
    // never true for the arguments the host passes; keeps the chains live
    if (s == -1.0) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

using namespace agb;

extern "C" agb_status agb_fp64_fma_peak(int iters, double* tflops, float* ms)
{
    if (!tflops || iters < 1) {
        set_error("agb_fp64_fma_peak: null output or iters < 1");
        return AGB_BADARG;
    }
    const int blocks = 4 * sm_count(), threads = 256;
    double* sink = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    agb_status rc = AGB_OK;
    float t = 0.0f;
    if (cudaMalloc(&sink, sizeof(double) * blocks * threads) != cudaSuccess ||
        cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        set_error(cudaGetErrorString(cudaGetLastError()));
        rc = AGB_CUDA;
    } else {
        k_fp64_fma<<<blocks, threads, 0, st>>>(sink, iters, 0.9999999, 1e-7);   // warm-up
        count_launch();
        cudaEventRecord(e0, st);
        k_fp64_fma<<<blocks, threads, 0, st>>>(sink, iters, 0.9999999, 1e-7);
        cudaEventRecord(e1, st);
        count_launch();
        cudaError_t e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error(cudaGetErrorString(e));
            rc = AGB_CUDA;
        } else {
            cudaEventElapsedTime(&t, e0, e1);
            const double flops = 2.0 * CHAINS * UNROLL * (double)iters * blocks * threads;
            *tflops = flops / (t * 1e-3) / 1e12;
            if (ms) *ms = t;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    if (sink) cudaFree(sink);
    return rc;
}
