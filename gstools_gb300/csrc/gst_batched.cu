// Batched randomization-method summation: many realizations, each with its
// own modes and its own point set of uneven size, in one persistent launch.
//
// The reference generates ensembles by looping in Python over seeds, one
// native summate call per realization (examples/01_random_field/
// 01_srf_ensemble.py; summate math src/gstools/field/generator.py:193-199).
// Here the whole ensemble is one step:
//
//   prepare (once per ensemble shape, host):
//     realization descriptors and a list of work tiles (realization, point
//     range) sorted by cost (modes x points, longest first) are uploaded into
//     the caller's workspace;
//   run (every step, asynchronous, no allocation -- capturable in a graph):
//     1. reset the work-queue counter,
//     2. pack every realization's modes into the mixed-precision table
//        (64-byte entries, each realization padded to whole mode tiles),
//     3. one persistent kernel (2 CTAs per SM) pulls tiles from the queue
//        with an atomic counter; per tile the points stay in registers and the
//        realization's mode tiles stream through shared memory by bulk (TMA)
//        copies, double-buffered on mbarriers (bounded waits).
//
// Arithmetic is the mixed-precision path (gst_mixed.cuh): exact turn
// reduction, SFU sin/cos, FP32 sums per 256-mode tile, FP64 across tiles.
// Tile shape (points per thread) is a template parameter; the Python layer
// times the variants on the real ensemble and keeps the fastest.
#include <algorithm>
#include <cstring>
#include <vector>

#include "gst_common.cuh"
#include "gst_mixed.cuh"

namespace gst {
namespace {

constexpr int kThreads = 256;
constexpr int kTileModes = 256;
constexpr int kEntryBytes = 64;
constexpr uint32_t kStageBytes = kTileModes * kEntryBytes;

__host__ __device__ __forceinline__ int64_t padded_modes(int64_t n) {
    return (n + kTileModes - 1) / kTileModes * kTileModes;
}

struct Item {            // one realization
    int64_t mode_off;    // first mode in the concatenated cov / z arrays
    int64_t n_modes;
    int64_t table_off;   // first entry in the packed table
    int64_t pt_off;      // first point in the concatenated pos / out arrays
    int64_t n_pts;
    int64_t pad;
};

struct Tile {
    int64_t item;
    int64_t pt_begin;    // relative to the realization's first point
};

struct Layout {
    size_t counter_off, items_off, tiles_off, table_off, shift_off, total;
    int64_t n_tiles, table_entries;
};

int points_per_tile(int variant) { return kThreads * (variant == 0 ? 2 : 4); }

int make_layout(int dim, int64_t n_items, const int64_t *modes, const int64_t *pts,
                int variant, Layout &l) {
    if (n_items < 0 || (n_items > 0 && (modes == nullptr || pts == nullptr)))
        return GST_ERR_INVALID_ARGUMENT;
    if (variant != 0 && variant != 1) return GST_ERR_INVALID_ARGUMENT;
    const int64_t tp = points_per_tile(variant);
    l.n_tiles = 0;
    l.table_entries = 0;
    for (int64_t r = 0; r < n_items; ++r) {
        if (modes[r] < 0 || pts[r] < 0) return GST_ERR_INVALID_ARGUMENT;
        l.n_tiles += ceil_div(pts[r], tp);
        l.table_entries += ceil_div(modes[r], kTileModes) * kTileModes;
    }
    if (l.n_tiles > 0x7fffffffLL) return GST_ERR_TOO_LARGE;
    l.counter_off = 0;
    l.items_off = 256;
    l.tiles_off = align_up(l.items_off + sizeof(Item) * n_items, 256);
    l.table_off = align_up(l.tiles_off + sizeof(Tile) * l.n_tiles, 256);
    // positions relative to each realization's first point (mixed path)
    int64_t total_pts = 0;
    for (int64_t r = 0; r < n_items; ++r) total_pts += pts[r];
    l.shift_off = align_up(l.table_off + static_cast<size_t>(l.table_entries) * kEntryBytes,
                           256);
    l.total = l.shift_off + sizeof(double) * static_cast<size_t>(dim > 0 ? dim : 0) *
                                static_cast<size_t>(total_pts);
    return GST_OK;
}

// Coordinate d of realization it's shift origin: its first point
// (gst_mixed.cuh, rotate_to_origin).
__device__ __forceinline__ double item_origin(const double *pos, int64_t total_pts,
                                              const Item &it, int d, int dim) {
    return (d < dim && it.n_pts > 0) ? origin_coord(pos + d * total_pts + it.pt_off)
                                     : 0.0;
}

// One thread per table entry of realization blockIdx.y; amplitudes rotated
// to the realization's first point.
__global__ void pack_batch_kernel(int dim, const Item *__restrict__ items,
                                  int64_t total_modes,
                                  const double *__restrict__ cov,
                                  const double *__restrict__ z1,
                                  const double *__restrict__ z2,
                                  const double *__restrict__ pos, int64_t total_pts,
                                  unsigned char *__restrict__ table) {
    const Item it = items[blockIdx.y];
    const int64_t padded = padded_modes(it.n_modes);
    const double x0[3] = {item_origin(pos, total_pts, it, 0, dim),
                          item_origin(pos, total_pts, it, 1, dim),
                          item_origin(pos, total_pts, it, 2, dim)};
    for (int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
         j < padded; j += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        double k[4] = {0.0, 0.0, 0.0, 0.0};
        double a1 = 0.0, a2 = 0.0;
        const double proj[3] = {0.0, 0.0, 0.0};
        if (j < it.n_modes) {
            for (int d = 0; d < dim; ++d) k[d] = cov[d * total_modes + it.mode_off + j];
            a1 = z1[it.mode_off + j];
            a2 = z2[it.mode_off + j];
            rotate_to_origin(k, dim, x0, a1, a2);
        }
        mixed_pack_entry(reinterpret_cast<float *>(table) + (it.table_off + j) * 16,
                         k, a1, a2, proj);
    }
}

// Positions relative to each realization's first point, into the
// workspace: realization blockIdx.y, grid-stride over its points.  (Done
// here rather than at the kernel's point loads, where the extra operands
// were measured to cost the summation 3.7 %.)
__global__ void shift_points_kernel(int dim, const Item *__restrict__ items,
                                    const double *__restrict__ pos, int64_t total_pts,
                                    double *__restrict__ shifted) {
    const Item it = items[blockIdx.y];
    for (int d = 0; d < dim; ++d) {
        const double x0 = item_origin(pos, total_pts, it, d, dim);
        const double *src = pos + d * total_pts + it.pt_off;
        double *dst = shifted + d * total_pts + it.pt_off;
        for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
             i < it.n_pts; i += static_cast<int64_t>(gridDim.x) * blockDim.x)
            dst[i] = src[i] - x0;
    }
}

struct BatchArgs {
    const Item *items;
    const Tile *tiles;
    int64_t n_tiles;
    unsigned int *counter;
    const unsigned char *table;
    const double *pos;
    int64_t total_pts;
    const double *scales;   // per realization, may be null (1.0)
    void *out;
    int out_f32;
    unsigned int *err;
};

template <int DIM, int P>
__global__ void __launch_bounds__(kThreads, 2) batched_kernel(const BatchArgs a) {
    __shared__ __align__(128) unsigned char stage[2][kStageBytes];
    __shared__ __align__(8) uint64_t full_bar[2];
    __shared__ int64_t s_tile;

    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(&full_bar[0], 1);
        mbar_init(&full_bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();

    uint64_t consumed = 0;  // mode tiles consumed by this CTA (phase tracking)
    bool ok = true;
    for (;;) {
        if (tid == 0) s_tile = atomicAdd(a.counter, 1u);
        __syncthreads();
        const int64_t t = s_tile;
        __syncthreads();
        if (t >= a.n_tiles || !ok) break;
        const Tile tile = a.tiles[t];
        const Item it = a.items[tile.item];

        double x[P][DIM];
        bool valid[P];
#pragma unroll
        for (int p = 0; p < P; ++p) {
            const int64_t i = tile.pt_begin + p * kThreads + tid;
            valid[p] = i < it.n_pts;
#pragma unroll
            for (int d = 0; d < DIM; ++d)
                x[p][d] = valid[p] ? a.pos[d * a.total_pts + it.pt_off + i] : 0.0;
        }
        MixedPoint<DIM> mp[P];
#pragma unroll
        for (int p = 0; p < P; ++p) mp[p] = mixed_split_point<DIM>(x[p]);
        double acc[P];
#pragma unroll
        for (int p = 0; p < P; ++p) acc[p] = 0.0;

        const int64_t n_mt = padded_modes(it.n_modes) / kTileModes;
        const unsigned char *src = a.table + it.table_off * kEntryBytes;
        if (tid == 0) {
            for (int64_t s = 0; s < 2 && s < n_mt; ++s) {
                const int slot = static_cast<int>((consumed + s) & 1);
                mbar_arrive_expect_tx(&full_bar[slot], kStageBytes);
                bulk_copy_g2s(stage[slot], src + s * kStageBytes, kStageBytes,
                              &full_bar[slot]);
            }
        }
        for (int64_t mt = 0; mt < n_mt; ++mt) {
            const uint64_t gidx = consumed + mt;
            const int slot = static_cast<int>(gidx & 1);
            const bool got = mbar_wait(&full_bar[slot],
                                       static_cast<uint32_t>((gidx >> 1) & 1), a.err);
            float accf[P];
#pragma unroll
            for (int p = 0; p < P; ++p) accf[p] = 0.0f;
            const float4 *e = reinterpret_cast<const float4 *>(stage[slot]);
#pragma unroll 2
            for (int jj = 0; jj < kTileModes; ++jj, e += 4) {
                const float4 qa = e[0];
                const float4 qb = e[1];
                const float qh[3] = {qa.x, qa.y, qa.z};
                const float ql[3] = {qb.x, qb.y, qb.z};
#pragma unroll
                for (int p = 0; p < P; ++p) {
                    float sn, cs;
                    mixed_sincos<DIM>(qh, ql, mp[p], &sn, &cs);
                    accf[p] = fmaf(qa.w, cs, fmaf(qb.w, sn, accf[p]));
                }
            }
#pragma unroll
            for (int p = 0; p < P; ++p) acc[p] += static_cast<double>(accf[p]);
            if (__syncthreads_or(!got)) {
                // mode tiles mt, mt + 1 may still be landing in shared
                // memory: drain them before the CTA exits
                if (tid == 0)
                    mbar_drain(full_bar, 2, gidx,
                               consumed + static_cast<uint64_t>(min(mt + 2, n_mt)),
                               a.err);
                ok = false;
                break;
            }
            if (tid == 0 && mt + 2 < n_mt) {
                mbar_arrive_expect_tx(&full_bar[slot], kStageBytes);
                bulk_copy_g2s(stage[slot], src + (mt + 2) * kStageBytes,
                              kStageBytes, &full_bar[slot]);
            }
        }
        consumed += n_mt;
        if (!ok) break;

        const double scale = a.scales ? a.scales[tile.item] : 1.0;
#pragma unroll
        for (int p = 0; p < P; ++p) {
            if (!valid[p]) continue;
            const int64_t o = it.pt_off + tile.pt_begin + p * kThreads + tid;
            if (a.out_f32)
                static_cast<float *>(a.out)[o] = static_cast<float>(scale * acc[p]);
            else
                static_cast<double *>(a.out)[o] = scale * acc[p];
        }
    }
}

template <int DIM>
cudaError_t launch_batched(int variant, int blocks, const BatchArgs &args,
                           cudaStream_t s) {
    if (variant == 0)
        batched_kernel<DIM, 2><<<blocks, kThreads, 0, s>>>(args);
    else
        batched_kernel<DIM, 4><<<blocks, kThreads, 0, s>>>(args);
    return cudaGetLastError();
}

}  // namespace
}  // namespace gst

extern "C" {

int gst_batch_workspace_size(int dim, int64_t n_items, const int64_t *mode_counts,
                             const int64_t *point_counts, int variant,
                             size_t *bytes) {
    if (bytes == nullptr) return GST_ERR_INVALID_ARGUMENT;
    if (dim < 1 || dim > 3) return GST_ERR_UNSUPPORTED_DIM;
    gst::Layout l;
    const int rc = gst::make_layout(dim, n_items, mode_counts, point_counts, variant, l);
    if (rc) return rc;
    *bytes = l.total;
    return GST_OK;
}

int gst_batch_prepare(int dim, int64_t n_items, const int64_t *mode_counts,
                      const int64_t *point_counts, int variant, void *workspace,
                      size_t workspace_bytes, void *stream) {
    using namespace gst;
    if (dim < 1 || dim > 3) return GST_ERR_UNSUPPORTED_DIM;
    Layout l;
    int rc = make_layout(dim, n_items, mode_counts, point_counts, variant, l);
    if (rc) return rc;
    if (workspace == nullptr || workspace_bytes < l.total) return GST_ERR_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(workspace) % 256 != 0) return GST_ERR_ALIGNMENT;
    if (current_device() < 0) return GST_ERR_NO_DEVICE;

    std::vector<unsigned char> host(l.table_off, 0);
    Item *items = reinterpret_cast<Item *>(host.data() + l.items_off);
    Tile *tiles = reinterpret_cast<Tile *>(host.data() + l.tiles_off);
    int64_t mode_off = 0, pt_off = 0, table_off = 0, nt = 0;
    const int64_t tp = points_per_tile(variant);
    std::vector<std::pair<int64_t, int64_t>> order;  // (cost, tile index)
    order.reserve(static_cast<size_t>(l.n_tiles));
    for (int64_t r = 0; r < n_items; ++r) {
        items[r] = Item{mode_off, mode_counts[r], table_off, pt_off,
                        point_counts[r], 0};
        const int64_t padded = ceil_div(mode_counts[r], kTileModes) * kTileModes;
        for (int64_t b = 0; b < point_counts[r]; b += tp) {
            tiles[nt] = Tile{r, b};
            order.emplace_back(padded * std::min(tp, point_counts[r] - b), nt);
            ++nt;
        }
        mode_off += mode_counts[r];
        pt_off += point_counts[r];
        table_off += padded;
    }
    // longest tiles first (LPT) so the queue ends with short work
    std::stable_sort(order.begin(), order.end(),
                     [](const auto &p, const auto &q) { return p.first > q.first; });
    std::vector<Tile> sorted(static_cast<size_t>(nt));
    for (int64_t i = 0; i < nt; ++i) sorted[i] = tiles[order[i].second];
    if (nt > 0) std::memcpy(tiles, sorted.data(), sizeof(Tile) * nt);

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    GST_TRY_CUDA(cudaMemcpyAsync(workspace, host.data(), host.size(),
                                 cudaMemcpyHostToDevice, s));
    GST_TRY_CUDA(cudaStreamSynchronize(s));
    return GST_OK;
}

int gst_batch_run(int dim, int64_t n_items, const int64_t *mode_counts,
                  const int64_t *point_counts, int variant, const double *cov,
                  const double *z_1, const double *z_2, const double *pos,
                  const double *scales, void *out, int out_type,
                  void *workspace, size_t workspace_bytes, void *stream) {
    using namespace gst;
    if (dim < 1 || dim > 3) return GST_ERR_UNSUPPORTED_DIM;
    if (out_type != GST_OUT_F64 && out_type != GST_OUT_F32)
        return GST_ERR_INVALID_ARGUMENT;
    Layout l;
    int rc = make_layout(dim, n_items, mode_counts, point_counts, variant, l);
    if (rc) return rc;
    int64_t total_modes = 0, total_pts = 0, max_padded = 0;
    for (int64_t r = 0; r < n_items; ++r) {
        total_modes += mode_counts[r];
        total_pts += point_counts[r];
        max_padded = std::max(max_padded, ceil_div(mode_counts[r], kTileModes) * kTileModes);
    }
    if (total_pts == 0) return GST_OK;
    if (workspace == nullptr || workspace_bytes < l.total || out == nullptr ||
        pos == nullptr)
        return GST_ERR_INVALID_ARGUMENT;
    if (total_modes > 0 && (cov == nullptr || z_1 == nullptr || z_2 == nullptr))
        return GST_ERR_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(workspace) % 256 != 0) return GST_ERR_ALIGNMENT;
    if (n_items > 65535) return GST_ERR_TOO_LARGE;
    if (current_device() < 0) return GST_ERR_NO_DEVICE;
    unsigned int *err = device_error_word();
    if (err == nullptr) return GST_ERR_CUDA;

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned char *ws = static_cast<unsigned char *>(workspace);
    GST_TRY_CUDA(cudaMemsetAsync(ws + l.counter_off, 0, sizeof(unsigned int), s));
    if (max_padded > 0) {
        const dim3 grid(static_cast<unsigned>(std::min<int64_t>(ceil_div(max_padded, 256), 64)),
                        static_cast<unsigned>(n_items));
        pack_batch_kernel<<<grid, 256, 0, s>>>(
            dim, reinterpret_cast<const Item *>(ws + l.items_off), total_modes, cov,
            z_1, z_2, pos, total_pts, ws + l.table_off);
        GST_TRY_CUDA(cudaGetLastError());
    }
    double *shifted = reinterpret_cast<double *>(ws + l.shift_off);
    {
        int64_t max_pts = 0;
        for (int64_t r = 0; r < n_items; ++r) max_pts = std::max(max_pts, point_counts[r]);
        const dim3 grid(static_cast<unsigned>(std::max<int64_t>(
                            1, std::min<int64_t>(ceil_div(max_pts, 256), 64))),
                        static_cast<unsigned>(n_items));
        shift_points_kernel<<<grid, 256, 0, s>>>(
            dim, reinterpret_cast<const Item *>(ws + l.items_off), pos, total_pts, shifted);
        GST_TRY_CUDA(cudaGetLastError());
    }
    BatchArgs args{};
    args.items = reinterpret_cast<const Item *>(ws + l.items_off);
    args.tiles = reinterpret_cast<const Tile *>(ws + l.tiles_off);
    args.n_tiles = l.n_tiles;
    args.counter = reinterpret_cast<unsigned int *>(ws + l.counter_off);
    args.table = ws + l.table_off;
    args.pos = shifted;
    args.total_pts = total_pts;
    args.scales = scales;
    args.out = out;
    args.out_f32 = out_type == GST_OUT_F32 ? 1 : 0;
    args.err = err;
    const int blocks = sm_count() * 2;
    cudaError_t e = cudaErrorInvalidValue;
    switch (dim) {
        case 1: e = launch_batched<1>(variant, blocks, args, s); break;
        case 2: e = launch_batched<2>(variant, blocks, args, s); break;
        case 3: e = launch_batched<3>(variant, blocks, args, s); break;
    }
    GST_TRY_CUDA(e);
    return GST_OK;
}

}  // extern "C"
