// Issue-rate probe for the roofline denominators of the product kernels: how many fused
// multiply-adds per second the SMs retire for one value type.  The products of libgsa do
// one FMA per real multiply-add (four per complex one); on GB300 the FP64 pipe retires far
// fewer of them per clock than the FP32 pipe, so FP64 products are bound by that pipe as
// well as by HBM.  A measurement aid for bench.py, not part of the library.
#include <cuda_runtime.h>
#include <stdint.h>

// Every thread runs 8 independent FMA chains of `iters` steps; x -> x * a + b with a just
// below 1 keeps the values finite.  The sum is stored only if it equals a value it cannot
// take, so nothing is written and nothing is folded away.
template <typename T>
__global__ void __launch_bounds__(256) fma_rate_kernel(T *out, int64_t iters, T a, T b) {
    T x[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = (T)(threadIdx.x + c) * (T)1e-3;
    for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = fma(x[c], a, b);
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) s += x[c];
    if (s == (T)-1.0) out[0] = s;
}

template <typename T>
static int probe(cudaStream_t s, int64_t iters, double *fma_per_s) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
    T *out = nullptr;
    if (cudaMallocAsync((void **)&out, sizeof(T), s) != cudaSuccess) return 2;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const unsigned blocks = (unsigned)sms * 8;  // 2048 threads per SM
    fma_rate_kernel<T><<<blocks, 256, 0, s>>>(out, iters / 8, (T)0.999999, (T)1e-6);  // warm-up
    cudaEventRecord(e0, s);
    fma_rate_kernel<T><<<blocks, 256, 0, s>>>(out, iters, (T)0.999999, (T)1e-6);
    cudaEventRecord(e1, s);
    int rc = cudaEventSynchronize(e1) == cudaSuccess ? 0 : 3;
    float ms = 0.f;
    if (!rc) rc = cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess ? 0 : 3;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(out, s);
    if (rc) return rc;
    *fma_per_s = (double)blocks * 256.0 * 8.0 * (double)iters / ((double)ms * 1e-3);
    return 0;
}

// dtype 0: float, 1: double.  Returns 0 on success; synchronizes the stream.
extern "C" int probe_fma_rate(void *stream, int dtype, int64_t iters, double *fma_per_s) {
    if (!fma_per_s || iters <= 0) return 4;
    if (dtype == 0) return probe<float>((cudaStream_t)stream, iters, fma_per_s);
    if (dtype == 1) return probe<double>((cudaStream_t)stream, iters, fma_per_s);
    return 4;
}
