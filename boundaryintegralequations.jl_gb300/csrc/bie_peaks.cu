// FMA-throughput probe behind bie_measure_peaks: the measured FP64 / FP32
// pipe peaks used as roofline denominators for the compute-bound assembly and
// operator kernels (the HBM and tensor-core peaks come from the copy / GEMM
// measurements of the deployment).
#include "bie_internal.h"

namespace bie {
namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;

template <typename T>
__global__ void __launch_bounds__(256) fma_chains(T *out, T a, T b) {
    T x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = (T)(threadIdx.x + c);
    for (int it = 0; it < kIters; ++it) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == (T)12345.678) out[threadIdx.x] = s;   // keeps the chains alive
}

template <typename T>
double time_fma(int sms, T *scratch, cudaStream_t st) {
    const int blocks = sms * 8, threads = 256;
    cudaEvent_t e0, e1;
    BIE_CUDA(cudaEventCreate(&e0));
    BIE_CUDA(cudaEventCreate(&e1));
    fma_chains<T><<<blocks, threads, 0, st>>>(scratch, (T)0.999999, (T)1e-7);   // warm-up
    BIE_CUDA(cudaGetLastError());
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        BIE_CUDA(cudaEventRecord(e0, st));
        fma_chains<T><<<blocks, threads, 0, st>>>(scratch, (T)0.999999, (T)1e-7);
        BIE_CUDA(cudaEventRecord(e1, st));
        BIE_CUDA(cudaEventSynchronize(e1));
        float ms;
        BIE_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        best = ms < best ? ms : best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double flops = 2.0 * kChains * kIters * (double)blocks * threads;
    return flops / (best * 1e-3);
}

}  // namespace

void measure_peaks(int device, bie_peaks &out) {
    BIE_CUDA(cudaSetDevice(device));
    int sms = 0;
    BIE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    cudaStream_t st;
    BIE_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    double *scratch = nullptr;
    BIE_CUDA(cudaMalloc(&scratch, 256 * sizeof(double)));
    out.fp64_flops = time_fma<double>(sms, scratch, st);
    out.fp32_flops = time_fma<float>(sms, reinterpret_cast<float *>(scratch), st);
    cudaFree(scratch);
    cudaStreamDestroy(st);
}

}  // namespace bie
