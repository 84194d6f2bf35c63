// Library-wide runtime pieces: version, status strings, per-device caches and
// the device error word that bounded waits report into.
#include <mutex>

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
// Freed scratch the library's pool keeps mapped for the next call.
constexpr uint64_t kScratchKeepBytes = 1ull << 30;
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

}  // extern "C"
