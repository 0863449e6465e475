// Issue-rate probe for the roofline denominators of the product kernels: how many fused
// multiply-adds per second the SMs retire for one value type.  The products of this
// library do one FMA per real multiply-add (four per complex one); on GB300 the FP64 pipe
// retires far fewer of them per clock than the FP32 pipe, so FP64 products are bound by
// that pipe as well as by HBM.  No counterpart in the reference.
#include "gsa_internal.cuh"

namespace gsa {

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
    int rc = check_cuda(cudaGetDevice(&dev), "probe: device");
    if (!rc) rc = check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "probe: SMs");
    if (rc) return rc;
    T *out = nullptr;
    rc = check_cuda(cudaMallocAsync((void **)&out, sizeof(T), s), "probe: scratch");
    if (rc) return rc;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const unsigned blocks = (unsigned)sms * 8;  // 2048 threads per SM
    fma_rate_kernel<T><<<blocks, 256, 0, s>>>(out, iters / 8, (T)0.999999, (T)1e-6);  // warm-up
    cudaEventRecord(e0, s);
    fma_rate_kernel<T><<<blocks, 256, 0, s>>>(out, iters, (T)0.999999, (T)1e-6);
    cudaEventRecord(e1, s);
    rc = check_cuda(cudaEventSynchronize(e1), "probe: run");
    float ms = 0.f;
    if (!rc) rc = check_cuda(cudaEventElapsedTime(&ms, e0, e1), "probe: time");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(out, s);
    if (rc) return rc;
    *fma_per_s = (double)blocks * 256.0 * 8.0 * (double)iters / ((double)ms * 1e-3);
    return GSA_OK;
}

}  // namespace gsa

extern "C" int gsa_probe_fma_rate(void *stream, int dtype, int64_t iters, double *fma_per_s) {
    using namespace gsa;
    if (!fma_per_s || iters <= 0) return fail(GSA_ERR_INVALID_ARG, "bad arguments");
    if (dtype == GSA_F32) return probe<float>((cudaStream_t)stream, iters, fma_per_s);
    if (dtype == GSA_F64) return probe<double>((cudaStream_t)stream, iters, fma_per_s);
    return fail(GSA_ERR_UNSUPPORTED, "probe: dtype must be F32 or F64");
}
