// Library-wide runtime pieces: version, status strings, per-device caches and
// the device error word that bounded waits report into.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "gst_common.cuh"

namespace {

__device__ unsigned int g_device_error_word;

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
int g_sm_count[kMaxDevices];
unsigned int *g_error_word[kMaxDevices];
cudaMemPool_t g_scratch_pool[kMaxDevices];
bool g_scratch_pool_tried[kMaxDevices];
cudaStream_t g_copy_stream[kMaxDevices];
// Freed scratch the library's pool keeps mapped for the next call (the
// largest single user, the sliced kriging variance, takes ~2.5 GB for
// 1000 conditions x 65 536 targets).
constexpr uint64_t kScratchKeepBytes = 4ull << 30;
thread_local cudaError_t g_last_cuda_error = cudaSuccess;

}  // namespace

namespace gst {

void note_cuda_error(cudaError_t err) { g_last_cuda_error = err; }

int current_device() {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (dev < 0 || dev >= kMaxDevices) return -1;
    return dev;
}

int sm_count() {
    const int dev = current_device();
    if (dev < 0) return 152;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (g_sm_count[dev] == 0) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) !=
                cudaSuccess ||
            n <= 0)
            n = 152;
        g_sm_count[dev] = n;
    }
    return g_sm_count[dev];
}

cudaStream_t copy_stream() {
    const int dev = current_device();
    if (dev < 0) return nullptr;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (g_copy_stream[dev] == nullptr) {
        cudaStream_t st = nullptr;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        g_copy_stream[dev] = st;
    }
    return g_copy_stream[dev];
}

cudaMemPool_t scratch_pool() {
    const int dev = current_device();
    if (dev < 0) return nullptr;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_pool_tried[dev]) {
        g_scratch_pool_tried[dev] = true;
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        if (cudaMemPoolCreate(&pool, &props) == cudaSuccess) {
            uint64_t keep = kScratchKeepBytes;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
            g_scratch_pool[dev] = pool;
        } else {
            cudaGetLastError();
        }
    }
    return g_scratch_pool[dev];
}

unsigned int *device_error_word() {
    const int dev = current_device();
    if (dev < 0) return nullptr;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (g_error_word[dev] == nullptr) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_device_error_word) != cudaSuccess)
            return nullptr;
        g_error_word[dev] = static_cast<unsigned int *>(p);
    }
    return g_error_word[dev];
}

}  // namespace gst

extern "C" {

int gst_version(void) { return 100; }

const char *gst_status_string(int status) {
    switch (status) {
        case GST_OK: return "ok";
        case GST_ERR_INVALID_ARGUMENT: return "invalid argument";
        case GST_ERR_UNSUPPORTED_DIM: return "unsupported dimension";
        case GST_ERR_CUDA: return "CUDA runtime error";
        case GST_ERR_ALIGNMENT: return "misaligned pointer";
        case GST_ERR_NO_DEVICE: return "no usable CUDA device";
        case GST_ERR_DEVICE_TIMEOUT: return "device-side wait timed out";
        case GST_ERR_TOO_LARGE: return "size exceeds the supported maximum";
        default: return "unknown status";
    }
}

int gst_last_cuda_error(void) { return static_cast<int>(g_last_cuda_error); }

int gst_read_device_error(void *stream, uint32_t *device_error) {
    if (device_error == nullptr) return GST_ERR_INVALID_ARGUMENT;
    if (gst::current_device() < 0) return GST_ERR_NO_DEVICE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    GST_TRY_CUDA(cudaStreamSynchronize(s));
    unsigned int word = 0;
    GST_TRY_CUDA(cudaMemcpyFromSymbol(&word, g_device_error_word,
                                      sizeof(word)));
    const unsigned int zero = 0;
    GST_TRY_CUDA(cudaMemcpyToSymbol(g_device_error_word, &zero, sizeof(zero)));
    *device_error = word;
    return GST_OK;
}

int gst_host_gather(int64_t n_arrays, const uint64_t *src, const int64_t *cols,
                    int64_t rows, double *dst, int64_t dst_cols, int threads) {
    if (n_arrays < 0 || rows < 0 || dst_cols < 0) return GST_ERR_INVALID_ARGUMENT;
    if (n_arrays == 0 || rows == 0 || dst_cols == 0) return GST_OK;
    if (src == nullptr || cols == nullptr || dst == nullptr) return GST_ERR_INVALID_ARGUMENT;
    // column offset of every array in a row of dst
    std::vector<int64_t> off(static_cast<size_t>(n_arrays) + 1, 0);
    for (int64_t a = 0; a < n_arrays; ++a) {
        if (cols[a] < 0 || (cols[a] > 0 && src[a] == 0)) return GST_ERR_INVALID_ARGUMENT;
        off[a + 1] = off[a] + cols[a];
    }
    if (off[n_arrays] != dst_cols) return GST_ERR_INVALID_ARGUMENT;
    const int64_t total = rows * dst_cols;   // elements of dst
    // Thread t fills the elements [t total / n, (t + 1) total / n) of dst
    // (row-major order): equal bytes per thread, contiguous writes.
    auto fill = [&](int64_t lo, int64_t hi) {
        while (lo < hi) {
            const int64_t row = lo / dst_cols, c = lo % dst_cols;
            const int64_t row_end = std::min(hi, (row + 1) * dst_cols);
            // the array holding column c
            int64_t a = std::upper_bound(off.begin(), off.end(), c) - off.begin() - 1;
            int64_t col = c;
            while (lo < row_end) {
                while (off[a + 1] <= col) ++a;   // skip arrays without columns
                const int64_t n = std::min(off[a + 1], col + (row_end - lo)) - col;
                const double *from = reinterpret_cast<const double *>(src[a]) +
                                     row * cols[a] + (col - off[a]);
                std::memcpy(dst + lo, from, static_cast<size_t>(n) * sizeof(double));
                lo += n;
                col += n;
            }
        }
    };
    int n = std::max(1, std::min(threads, 64));
    if (total * static_cast<int64_t>(sizeof(double)) < (4 << 20)) n = 1;
    if (n == 1) {
        fill(0, total);
        return GST_OK;
    }
    std::vector<std::thread> pool;
    pool.reserve(static_cast<size_t>(n));
    for (int t = 0; t < n; ++t)
        pool.emplace_back(fill, total * t / n, total * (t + 1) / n);
    for (auto &th : pool) th.join();
    return GST_OK;
}

}  // extern "C"
