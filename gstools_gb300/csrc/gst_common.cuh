// Shared device helpers and host plumbing for the gstools_gb300 kernels.
//
// Everything here is written for sm_103a: mbarrier-tracked bulk copies
// (cp.async.bulk, the TMA engine's untiled form) stage packed mode tables in
// shared memory, and every wait on an mbarrier is bounded in time so a lost
// transaction can never hang the GPU -- the kernel records
// GST_ERR_DEVICE_TIMEOUT in a device error word and returns.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gstools_gb300.h"

#define GST_TRY_CUDA(expr)                                  \
    do {                                                    \
        cudaError_t gst_err_ = (expr);                      \
        if (gst_err_ != cudaSuccess) {                      \
            ::gst::note_cuda_error(gst_err_);               \
            return GST_ERR_CUDA;                            \
        }                                                   \
    } while (0)

namespace gst {

// ------------------------------------------------------------------ host --

// Remembers the last CUDA error seen by an entry point (for diagnostics).
void note_cuda_error(cudaError_t err);

// Streaming multiprocessors of the current device (cached per device).
int sm_count();

// Address of the per-device error word that bounded waits report into.
unsigned int *device_error_word();

// Current device ordinal, or -1 with GST_ERR_NO_DEVICE semantics.
int current_device();

// The library's stream-ordered memory pool on the current device (created
// on first use; it keeps up to 1 GiB of freed scratch mapped, where the
// default pool unmaps it at every synchronisation), or null.
cudaMemPool_t scratch_pool();

// A non-blocking stream of the current device for device-to-host copies
// that overlap the library's kernels (created on first use), or null.
cudaStream_t copy_stream();

// Mixed-precision summate of one unstructured point set (gst_batched.cu):
// points sorted spatially and modes by |k|_1, amplitude-phase form, per-warp
// origins; out (n_pts) float32 (out_f32) or float64, scaled by `scale`.
int summate_mixed_sorted(int dim, int64_t n_modes, int64_t n_pts, const double *cov,
                         const double *z1, const double *z2, const double *pos,
                         void *out, int out_f32, double scale, cudaStream_t s);
// When gst_summate_mixed takes that path: at most kSortedMaxModes modes and
// at least kSortedMinWork mode-points, or, in 2-D and 3-D, at least
// kSortedMinWorkPts mode-points over at least kSortedMinPts points (measured
// crossovers: 2-D and 3-D sums of 4e8 mode-points over 2e5+ points run
// 10-20 % faster sorted; fewer points with many modes, and 1-D, run faster
// pointwise).
constexpr double kSortedMinWork = 1e9;
constexpr double kSortedMinWorkPts = 4e8;
constexpr int64_t kSortedMinPts = 200000;
constexpr int64_t kSortedMaxModes = 16384;

// Stream-ordered scratch allocation that always frees on the same stream.
struct StreamScratch {
    void *ptr = nullptr;
    cudaStream_t stream = nullptr;
    ~StreamScratch() {
        if (ptr) cudaFreeAsync(ptr, stream);
    }
    cudaError_t alloc(size_t bytes, cudaStream_t s) {
        stream = s;
        if (bytes == 0) return cudaSuccess;
        cudaMemPool_t pool = scratch_pool();
        if (pool != nullptr) return cudaMallocFromPoolAsync(&ptr, bytes, pool, s);
        return cudaMallocAsync(&ptr, bytes, s);
    }
};

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Device error codes ORed into the error word.
constexpr unsigned int kErrWaitTimeout = 1u;

// ---------------------------------------------------------------- device --

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(count)
                 : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar,
                                                      uint32_t bytes) {
    asm volatile(
        "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
            smem_addr(bar)),
        "r"(bytes)
        : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t global_timer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Upper bound on any single wait (nanoseconds).  Every phase a kernel waits
// for completes within microseconds when the hardware is healthy.
constexpr uint64_t kWaitLimitNs = 2000000000ull;

__device__ __forceinline__ bool mbar_try(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// try_wait with a suspend-time hint: the thread sleeps in hardware for up
// to about `hint_ns` while the phase is incomplete.
__device__ __forceinline__ bool mbar_try_hint(uint64_t *bar, uint32_t parity,
                                              uint32_t hint_ns) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity), "r"(hint_ns)
        : "memory");
    return ok != 0;
}

// Waits for `parity` of `bar`; gives up after kWaitLimitNs, records the
// timeout in *err and returns false.  try_wait suspends the thread in
// hardware between checks, so waiting warps do not steal issue slots.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity,
                                          unsigned int *err) {
    if (mbar_try(bar, parity)) return true;
    const uint64_t t0 = global_timer_ns();
    for (uint32_t it = 1;; ++it) {
        if (mbar_try(bar, parity)) return true;
        if ((it & 15u) == 0u && global_timer_ns() - t0 > kWaitLimitNs) {
            atomicOr(err, kErrWaitTimeout);
            return false;
        }
    }
}

// After a failed wait: waits (each bounded like mbar_wait) for every bulk
// copy still in flight into this CTA's ring of `n_stages` barriers -- the
// global stage indices [first, last), stage u on barrier u % n_stages with
// parity (u / n_stages) & 1 -- so that the CTA does not exit while the copy
// engine still writes into its shared memory.  One thread calls it.
__device__ __forceinline__ void mbar_drain(uint64_t *bars, int n_stages,
                                           uint64_t first, uint64_t last,
                                           unsigned int *err) {
    for (uint64_t u = first; u < last; ++u)
        mbar_wait(&bars[u % n_stages],
                  static_cast<uint32_t>((u / n_stages) & 1u), err);
}

// Bulk (TMA) copy global -> shared, completion signalled on `bar` as
// transaction bytes.  Both addresses 16-byte aligned, bytes % 16 == 0.
__device__ __forceinline__ void bulk_copy_g2s(void *smem_dst,
                                              const void *gmem_src,
                                              uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1], %2, [%3];" ::"r"(smem_addr(smem_dst)),
        "l"(gmem_src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Round-to-12-significant-bits split used by the mixed-precision kernels:
// v ~= hi + lo with hi carrying at most 12 significant bits, so the product
// of two such `hi` values is exact in FP32.
__device__ __forceinline__ float split_hi12(double v) {
    const float f = static_cast<float>(v);
    return __uint_as_float(__float_as_uint(f) & 0xFFFFF000u);
}

}  // namespace gst
