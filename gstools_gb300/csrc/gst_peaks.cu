// Throughput probes for the roofline denominators the driver does not
// measure: FP32 FMA, FP64 FMA and SFU sin/cos issue rates on this GPU.
// Each probe runs many independent dependency chains per thread so the
// pipe, not latency, limits it; the caller times the launch with CUDA events.
#include "gst_common.cuh"

namespace gst {
namespace {

constexpr int kChains = 8;
constexpr int kUnroll = 16;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) probe_f32_fma(int64_t iters,
                                                          float *sink) {
    float a[kChains];
    const float m = 1.0f + 1e-7f * threadIdx.x, c = 1e-8f;
#pragma unroll
    for (int i = 0; i < kChains; ++i) a[i] = threadIdx.x * 1e-3f + i;
    for (int64_t it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
#pragma unroll
            for (int i = 0; i < kChains; ++i) a[i] = fmaf(a[i], m, c);
    }
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < kChains; ++i) s += a[i];
    if (s == 12345.0f) sink[threadIdx.x] = s;
}

__global__ void __launch_bounds__(kThreads) probe_f64_fma(int64_t iters,
                                                          float *sink) {
    double a[kChains];
    const double m = 1.0 + 1e-15 * threadIdx.x, c = 1e-16;
#pragma unroll
    for (int i = 0; i < kChains; ++i) a[i] = threadIdx.x * 1e-3 + i;
    for (int64_t it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
#pragma unroll
            for (int i = 0; i < kChains; ++i) a[i] = fma(a[i], m, c);
    }
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < kChains; ++i) s += a[i];
    if (s == 12345.0) sink[threadIdx.x] = static_cast<float>(s);
}

__global__ void __launch_bounds__(kThreads) probe_sfu_sin(int64_t iters,
                                                          float *sink) {
    float a[kChains];
#pragma unroll
    for (int i = 0; i < kChains; ++i) a[i] = threadIdx.x * 1e-3f + 0.1f * i;
    for (int64_t it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
#pragma unroll
            for (int i = 0; i < kChains; ++i) a[i] = __sinf(a[i]);
    }
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < kChains; ++i) s += a[i];
    if (s == 12345.0f) sink[threadIdx.x] = s;
}

}  // namespace
}  // namespace gst

extern "C" int gst_peak_probe(int kind, int64_t iters, float *sink,
                              double *ops_per_launch, void *stream) {
    if (iters <= 0 || sink == nullptr || ops_per_launch == nullptr)
        return GST_ERR_INVALID_ARGUMENT;
    if (gst::current_device() < 0) return GST_ERR_NO_DEVICE;
    const int blocks = gst::sm_count() * 8;
    const double per_thread =
        static_cast<double>(iters) * gst::kUnroll * gst::kChains;
    const double threads = static_cast<double>(blocks) * gst::kThreads;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (kind) {
        case 0:  // FP32 FMA: 2 flops each
            gst::probe_f32_fma<<<blocks, gst::kThreads, 0, s>>>(iters, sink);
            *ops_per_launch = 2.0 * per_thread * threads;
            break;
        case 1:  // FP64 FMA: 2 flops each
            gst::probe_f64_fma<<<blocks, gst::kThreads, 0, s>>>(iters, sink);
            *ops_per_launch = 2.0 * per_thread * threads;
            break;
        case 2:  // SFU sin.approx: 1 op each
            gst::probe_sfu_sin<<<blocks, gst::kThreads, 0, s>>>(iters, sink);
            *ops_per_launch = per_thread * threads;
            break;
        default:
            return GST_ERR_INVALID_ARGUMENT;
    }
    GST_TRY_CUDA(cudaGetLastError());
    return GST_OK;
}
