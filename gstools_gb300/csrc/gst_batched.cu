// Batched randomization-method summation: many realizations, each with its
// own modes and its own point set of uneven size, in one persistent launch;
// and the mixed-precision summate of one large unstructured point set, which
// runs as a batch of one.
//
// The reference generates ensembles by looping in Python over seeds, one
// native summate call per realization (examples/01_random_field/
// 01_srf_ensemble.py; summate math src/gstools/field/generator.py:193-199).
// Here the whole ensemble is one step:
//
//   prepare (once per ensemble shape, host):
//     realization descriptors, sort segments, and a list of work tiles
//     (realization, point range) sorted by cost (modes x points, longest
//     first) are uploaded into the caller's workspace;
//   run (every step, asynchronous, no allocation -- capturable in a graph):
//     1. reset the work-queue counter;
//     2. pack every realization's modes into the mixed-precision table, in
//        ascending order of |k|_1 (a stable bucket sort per realization),
//        with the largest |k|_1 of every 32-mode chunk;
//     3. sort every realization's points spatially: a stable counting sort
//        on a 4096-cell Morton grid over the realization's bounding box, in
//        segments of 4096 points (segment bounding boxes, segment
//        histograms, one column scan per realization, segment scatters), so
//        that a work tile -- consecutive sorted points -- is compact;
//     4. one persistent warp-specialised kernel: a producer warp pulls work
//        items from the queue with an atomic counter and streams their mode
//        stages through a ring of shared-memory slots by bulk (TMA) copies,
//        each slot tagged with its (item, stage); eight consumer warps work
//        through the ring on full / empty mbarriers (bounded waits) with no
//        CTA-wide barrier, each on its own 32 P points.
//
// Arithmetic (amplitude-phase form).  z1 cos(theta) + z2 sin(theta) =
// A cos(theta - phi) with A = hypot(z1, z2), phi = atan2(z2, z1): one SFU
// cosine per mode and point instead of a sine and a cosine.  Phases are in
// turns, q = k / 2 pi.  The pack kernel reduces psi0 = phi / 2 pi - <q, x0>
// modulo 1 (x0 the realization's first point; <q, x0> in FP64).  Each warp
// takes the centre x_W of the bounding box of its 32 P points (consecutive
// in the sorted order, so close together) as origin; at every stage the warp
// reduces its offsets psi_W = psi0 - <q, x_W> (mod 1) once per mode with the
// exact split turn reduction (gst_mixed.cuh), so the phase of a point
// x = x0 + x_W + x'' is <q, x''> - psi_W.  Per 32-mode chunk (modes sorted
// by |k|_1), warp-uniformly:
//   * fast chunks -- the chunk's largest |k|_1 times the warp's half extent
//     is at most kFastBound radians: the phase <k, x''> - 2 pi psi_W is an
//     FP32 FMA chain of magnitude <= kFastBound + pi fed to __cosf (error
//     at most about 4e-7 + 4e-7 |arg| radians per mode and point);
//   * other chunks -- the exact split turn reduction of <q, x''> - psi_W.
// FP32 sums per stage, FP64 across stages.  Points per thread, modes per
// stage, CTAs per SM and ring depth are template parameters (variants); the
// Python layer times the variants on the real ensemble and keeps the
// fastest.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "gst_common.cuh"
#include "gst_mixed.cuh"

namespace gst {
namespace {

constexpr int kConsumerWarps = 8;
constexpr int kThreads = (kConsumerWarps + 1) * 32;   // + one producer warp
constexpr int kEntryFloats = 16;
constexpr int kEntryBytes = kEntryFloats * 4;
constexpr int kChunk = 32;          // modes per |k|_1 maximum (one warp pass)
constexpr int kModeBuckets = 128;
constexpr int kPackThreads = 256;
constexpr int kSortThreads = 1024;
constexpr int kScatterThreads = 512;
constexpr int kCells = 4096;        // Morton cells of the point sort
constexpr int kSegPoints = 4096;    // points per sort segment
// Largest |<k, x''>| (radians) a fast chunk may see: the FP32 phase error
// grows with it (see the header comment).  On the 512-realization Matern
// ensemble, bounds of 8 / 12 / 16 / 24 gave 17.5 / 16.5 / 15.7 / 15.1 ms
// at 6.7e-7 / 6.4e-7 / 6.5e-7 / 7.1e-7 sigma RMS against the FP64 oracle:
// 16 keeps the worst-case term error below 1e-5 rad at no measured cost in
// accuracy.
#ifndef GST_FAST_BOUND
#define GST_FAST_BOUND 16.0f
#endif
constexpr float kFastBound = GST_FAST_BOUND;

// Kernel shapes: points per consumer thread, modes per stage, CTAs per SM,
// ring slots.  A tile is 8 warps x 32 lanes x points.
struct Shape {
    int points, modes, ctas, ring;
};
constexpr Shape kShapes[] = {
    {2, 256, 2, 4},   // 0: 512-point tiles
    {4, 256, 2, 4},   // 1: 1024-point tiles
    {2, 256, 3, 3},   // 2: 512-point tiles, 3 CTAs per SM
    {2, 128, 3, 4},   // 3: 512-point tiles, 128-mode stages
    {1, 256, 4, 2},   // 4: 256-point tiles, 4 CTAs per SM
    {4, 128, 2, 6},   // 5: 1024-point tiles, 128-mode stages, deep ring
};
constexpr int kNumShapes = sizeof(kShapes) / sizeof(kShapes[0]);
// the shape of the single-call path
constexpr int kSingleShape = 2;

__host__ __device__ __forceinline__ int64_t padded_modes(int64_t n, int w) {
    return (n + w - 1) / w * w;
}

inline int64_t tile_points(int v) {
    return static_cast<int64_t>(kConsumerWarps) * 32 * kShapes[v].points;
}

struct Item {            // one realization
    int64_t mode_off;    // first mode in the concatenated cov / z arrays
    int64_t n_modes;
    int64_t table_off;   // first entry in the packed table
    int64_t pt_off;      // first point in the concatenated pos / out arrays
    int64_t n_pts;
    int64_t seg_off;     // first sort segment
    int64_t n_seg;
    int64_t pad;
};

struct Tile {
    int64_t item;
    int64_t pt_begin;    // relative to the realization's first point
};

struct Seg {             // kSegPoints points of one realization
    int64_t item;
    int64_t begin;       // relative to the realization's first point
};

struct Layout {
    size_t counter_off, items_off, tiles_off, segs_off, table_off, kmax_off, box_off,
        hist_off, sorted_off, perm_off, total;
    int64_t n_tiles, table_entries, n_seg;
};

int make_layout(int dim, int64_t n_items, const int64_t *modes, const int64_t *pts,
                int variant, Layout &l) {
    if (n_items < 0 || (n_items > 0 && (modes == nullptr || pts == nullptr)))
        return GST_ERR_INVALID_ARGUMENT;
    if (variant < 0 || variant >= kNumShapes) return GST_ERR_INVALID_ARGUMENT;
    const int64_t tp = tile_points(variant);
    const int w = kShapes[variant].modes;
    l.n_tiles = 0;
    l.table_entries = 0;
    l.n_seg = 0;
    int64_t total_pts = 0;
    for (int64_t r = 0; r < n_items; ++r) {
        if (modes[r] < 0 || pts[r] < 0) return GST_ERR_INVALID_ARGUMENT;
        if (pts[r] > 0x7fffffffLL) return GST_ERR_TOO_LARGE;
        l.n_tiles += ceil_div(pts[r], tp);
        l.n_seg += ceil_div(pts[r], kSegPoints);
        l.table_entries += padded_modes(modes[r], w);
        total_pts += pts[r];
    }
    if (l.n_tiles > 0x7fffffffLL || l.n_seg > 0x7fffffffLL) return GST_ERR_TOO_LARGE;
    l.counter_off = 0;
    l.items_off = 256;
    l.tiles_off = align_up(l.items_off + sizeof(Item) * n_items, 256);
    l.segs_off = align_up(l.tiles_off + sizeof(Tile) * l.n_tiles, 256);
    l.table_off = align_up(l.segs_off + sizeof(Seg) * l.n_seg, 256);
    l.kmax_off = align_up(l.table_off + static_cast<size_t>(l.table_entries) * kEntryBytes,
                          256);
    l.box_off = align_up(l.kmax_off + sizeof(float) * (l.table_entries / kChunk), 256);
    l.hist_off = align_up(l.box_off + sizeof(double) * 6 * l.n_seg, 256);
    l.sorted_off = align_up(l.hist_off + sizeof(unsigned) * kCells * l.n_seg, 256);
    l.perm_off = align_up(l.sorted_off + sizeof(double) *
                                             static_cast<size_t>(dim > 0 ? dim : 0) *
                                             static_cast<size_t>(total_pts),
                          256);
    l.total = l.perm_off + sizeof(int32_t) * static_cast<size_t>(total_pts);
    return GST_OK;
}

// Coordinate d of realization it's origin: its first point.
__device__ __forceinline__ double item_origin(const double *pos, int64_t total_pts,
                                              const Item &it, int d, int dim) {
    return (d < dim && it.n_pts > 0) ? origin_coord(pos + d * total_pts + it.pt_off)
                                     : 0.0;
}

__device__ __forceinline__ unsigned lanemask_lt() {
    return (1u << (threadIdx.x & 31)) - 1u;
}

__device__ __forceinline__ void mbar_arrive_local(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

// ------------------------------------------------------------ mode packing --

__device__ __forceinline__ unsigned mode_bucket(double key) {
    if (!(key > 0.0)) return 0u;   // zero modes (and NaN) first
    const int b = static_cast<int>(floor(log2(key) * 4.0)) + kModeBuckets / 2;
    return static_cast<unsigned>(min(max(b, 1), kModeBuckets - 1));
}

__device__ __forceinline__ double mode_key(int dim, const double *cov,
                                           int64_t total_modes, int64_t m) {
    double s = 0.0;
    for (int d = 0; d < dim; ++d) s += fabs(cov[d * total_modes + m]);
    return s;
}

// Table entry (16 floats) of one mode:
//   k0 k1 k2 A | qh0 qh1 qh2 psi0 | ql0 ql1 ql2 0 | 0 0 0 0
// k in FP32 (radians per unit, the fast path), q = k / 2 pi split into a
// 12-significant-bit head and an FP32 tail (the exact path), A = hypot(z1,
// z2), psi0 = atan2(z2, z1) / 2 pi - <q, x0> reduced to [-1/2, 1/2]: the
// dot product and its reduction in FP64, atan2 and hypot in FP32 (their
// results are rounded to FP32 in the table anyway).
__device__ void write_entry(float *e, int dim, const double *cov,
                            int64_t total_modes, int64_t m, const double *z1,
                            const double *z2, const double (&x0)[3]) {
    constexpr double kInv2Pi = 0.15915494309189533576888376337251436;
    double k[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < dim; ++d) k[d] = cov[d * total_modes + m];
    const double a1 = z1[m], a2 = z2[m];
    double t = 0.0;
    for (int d = 0; d < dim; ++d) t += (k[d] * kInv2Pi) * x0[d];
    t -= rint(t);
    const float phi = atan2f(static_cast<float>(a2), static_cast<float>(a1)) *
                      static_cast<float>(kInv2Pi);
    double psi = static_cast<double>(phi) - t;
    psi -= rint(psi);
    for (int d = 0; d < 3; ++d) {
        const double q = k[d] * kInv2Pi;
        const float qh = split_hi12(q);
        e[d] = static_cast<float>(k[d]);
        e[4 + d] = qh;
        e[8 + d] = static_cast<float>(q - static_cast<double>(qh));
    }
    e[3] = hypotf(static_cast<float>(a1), static_cast<float>(a2));
    e[7] = static_cast<float>(psi);
    for (int d = 11; d < 16; ++d) e[d] = 0.0f;
}

// One CTA per realization: stable bucket sort of its modes by |k|_1, the
// table entries in that order (zero entries up to the stage padding), and
// the largest FP32 |k|_1 of every 32-entry chunk (zeroed first, then raised
// by every entry written; the CTA's barriers order the zeroing before).
__global__ void __launch_bounds__(kPackThreads)
    pack_batch_kernel(int dim, const Item *__restrict__ items, int64_t total_modes,
                      const double *__restrict__ cov, const double *__restrict__ z1,
                      const double *__restrict__ z2, const double *__restrict__ pos,
                      int64_t total_pts, int stage_modes, float *__restrict__ table,
                      float *__restrict__ kmax) {
    __shared__ unsigned int hist[kModeBuckets];
    __shared__ unsigned int s_base[kPackThreads];
    const Item it = items[blockIdx.x];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t padded = padded_modes(it.n_modes, stage_modes);
    const double x0[3] = {item_origin(pos, total_pts, it, 0, dim),
                          item_origin(pos, total_pts, it, 1, dim),
                          item_origin(pos, total_pts, it, 2, dim)};
    float *kmax_r = kmax + it.table_off / kChunk;   // this realization's chunks
    for (int b = tid; b < kModeBuckets; b += kPackThreads) hist[b] = 0u;
    for (int64_t c = tid; c < padded / kChunk; c += kPackThreads) kmax_r[c] = 0.0f;
    __syncthreads();
    for (int64_t j = tid; j < it.n_modes; j += kPackThreads)
        atomicAdd(&hist[mode_bucket(mode_key(dim, cov, total_modes, it.mode_off + j))], 1u);
    __syncthreads();
    if (warp == 0) {   // exclusive scan, 4 buckets per lane
        unsigned v[4], sum = 0;
        for (int i = 0; i < 4; ++i) {
            v[i] = hist[lane * 4 + i];
            sum += v[i];
        }
        unsigned incl = sum;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned n = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += n;
        }
        unsigned run = incl - sum;
        for (int i = 0; i < 4; ++i) {
            hist[lane * 4 + i] = run;
            run += v[i];
        }
    }
    __syncthreads();
    float *base_e = table + it.table_off * kEntryFloats;
    for (int64_t c0 = 0; c0 < it.n_modes; c0 += kPackThreads) {
        const int64_t j = c0 + tid;
        const bool valid = j < it.n_modes;
        const unsigned b = valid ? mode_bucket(mode_key(dim, cov, total_modes,
                                                        it.mode_off + j))
                                 : 0xffffffffu;
        const unsigned peers = __match_any_sync(0xffffffffu, b);
        const int leader = __ffs(peers) - 1;
        const unsigned rank = __popc(peers & lanemask_lt());
        // warps claim their buckets' slots in warp order: stable
        for (int w = 0; w < kPackThreads / 32; ++w) {
            if (warp == w && valid && lane == leader) {
                s_base[tid] = hist[b];
                hist[b] += __popc(peers);
            }
            __syncthreads();
        }
        if (valid) {
            const unsigned dst = s_base[warp * 32 + leader] + rank;
            float *e = base_e + static_cast<int64_t>(dst) * kEntryFloats;
            write_entry(e, dim, cov, total_modes, it.mode_off + j, z1, z2, x0);
            // the chunk maximum of the FP32 |k|_1 (non-negative floats order
            // like their bit patterns, so an integer maximum; order-free)
            const float k1 = fabsf(e[0]) + fabsf(e[1]) + fabsf(e[2]);
            atomicMax(reinterpret_cast<int *>(kmax_r + dst / kChunk), __float_as_int(k1));
        }
        __syncthreads();
    }
    for (int64_t j = it.n_modes + tid; j < padded; j += kPackThreads) {
        float *e = base_e + j * kEntryFloats;
        for (int i = 0; i < kEntryFloats; ++i) e[i] = 0.0f;
    }
}

// -------------------------------------------------------------- point sort --
//
// A stable counting sort of every realization's points by the Morton cell
// (4096 cells over its bounding box) in segments of kSegPoints points:
// segment bounding boxes; per segment a cell histogram; per realization one
// CTA turns its segments' histograms into start offsets (cells in Morton
// order, segments in order within a cell); each segment scatters its points
// in order.  With `segs` null there is one realization and segment s starts
// at its point s kSegPoints.

__device__ __forceinline__ unsigned morton_key(int dim, const int (&c)[3]) {
    unsigned key = 0u;
    if (dim == 1) return static_cast<unsigned>(c[0]);
    if (dim == 2) {
        for (int b = 0; b < 6; ++b)
            key |= (((c[0] >> b) & 1u) << (2 * b)) | (((c[1] >> b) & 1u) << (2 * b + 1));
        return key;
    }
    for (int b = 0; b < 4; ++b)
        key |= (((c[0] >> b) & 1u) << (3 * b)) | (((c[1] >> b) & 1u) << (3 * b + 1)) |
               (((c[2] >> b) & 1u) << (3 * b + 2));
    return key;
}

__device__ __forceinline__ int cells_per_axis(int dim) {
    return dim == 1 ? kCells : (dim == 2 ? 64 : 16);
}

__device__ __forceinline__ Seg seg_of(const Seg *segs, int64_t s) {
    return segs ? segs[s] : Seg{0, s * kSegPoints};
}

__global__ void __launch_bounds__(256)
    seg_box_kernel(int dim, const Item *__restrict__ items, const Seg *__restrict__ segs,
                   const double *__restrict__ pos, int64_t total_pts,
                   double *__restrict__ box) {
    __shared__ double s_lo[8][3], s_hi[8][3];
    const Seg sg = seg_of(segs, blockIdx.x);
    const Item it = items[sg.item];
    const int64_t i1 = min(sg.begin + kSegPoints, it.n_pts);
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = sg.begin + threadIdx.x; i < i1; i += 256)
        for (int d = 0; d < dim; ++d) {
            const double v = pos[d * total_pts + it.pt_off + i];
            lo[d] = fmin(lo[d], v);
            hi[d] = fmax(hi[d], v);
        }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int d = 0; d < dim; ++d) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[d] = fmin(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
            hi[d] = fmax(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
        }
        if (lane == 0) {
            s_lo[warp][d] = lo[d];
            s_hi[warp][d] = hi[d];
        }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int d = threadIdx.x;
        double l = INFINITY, h = -INFINITY;
        if (d < dim)
            for (int w = 0; w < 8; ++w) {
                l = fmin(l, s_lo[w][d]);
                h = fmax(h, s_hi[w][d]);
            }
        box[blockIdx.x * 6 + d] = l;
        box[blockIdx.x * 6 + 3 + d] = h;
    }
}

// The realization's bounding box from its segments' boxes, and the cell
// scale of every axis, into s_lo / s_inv: computed by one whole warp (lanes
// stride over the segments), lane 0 stores.
__device__ __forceinline__ void item_cells_warp(int dim, const Item &it, const double *box,
                                                double *s_lo, double *s_inv) {
    const int lane = threadIdx.x & 31;
    const int cpa = cells_per_axis(dim);
    for (int d = 0; d < 3; ++d) {
        double l = INFINITY, h = -INFINITY;
        if (d < dim)
            for (int64_t s = lane; s < it.n_seg; s += 32) {
                l = fmin(l, box[(it.seg_off + s) * 6 + d]);
                h = fmax(h, box[(it.seg_off + s) * 6 + 3 + d]);
            }
        for (int o = 16; o > 0; o >>= 1) {
            l = fmin(l, __shfl_xor_sync(0xffffffffu, l, o));
            h = fmax(h, __shfl_xor_sync(0xffffffffu, h, o));
        }
        const double ext = h - l;
        if (lane == 0) {
            s_lo[d] = l;
            s_inv[d] = (d < dim && ext > 0.0 && isfinite(ext)) ? cpa / ext : 0.0;
        }
    }
}

// Morton cell of the point whose first coordinate is at p (coordinate d at
// p[d * stride]).
__device__ __forceinline__ unsigned point_cell(int dim, const double *p, int64_t stride,
                                               const double (&lo)[3],
                                               const double (&inv)[3]) {
    const int cpa = cells_per_axis(dim);
    int c[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) {
        const double f = (p[d * stride] - lo[d]) * inv[d];
        c[d] = (f >= 0.0) ? min(static_cast<int>(f), cpa - 1) : 0;  // NaN -> 0
    }
    return morton_key(dim, c);
}

__global__ void __launch_bounds__(kSortThreads)
    seg_hist_kernel(int dim, const Item *__restrict__ items, const Seg *__restrict__ segs,
                    const double *__restrict__ pos, int64_t total_pts,
                    const double *__restrict__ box, unsigned *__restrict__ hist) {
    __shared__ unsigned h[kCells];
    __shared__ double s_lo[3], s_inv[3];
    const Seg sg = seg_of(segs, blockIdx.x);
    const Item it = items[sg.item];
    if (threadIdx.x < 32) item_cells_warp(dim, it, box, s_lo, s_inv);
    for (int c = threadIdx.x; c < kCells; c += kSortThreads) h[c] = 0u;
    __syncthreads();
    const double lo[3] = {s_lo[0], s_lo[1], s_lo[2]};
    const double inv[3] = {s_inv[0], s_inv[1], s_inv[2]};
    const int64_t i1 = min(sg.begin + kSegPoints, it.n_pts);
    for (int64_t i = sg.begin + threadIdx.x; i < i1; i += kSortThreads)
        atomicAdd(&h[point_cell(dim, pos + it.pt_off + i, total_pts, lo, inv)], 1u);
    __syncthreads();
    unsigned *dst = hist + static_cast<int64_t>(blockIdx.x) * kCells;
    for (int c = threadIdx.x; c < kCells; c += kSortThreads) dst[c] = h[c];
}

// One CTA per realization: the start offset of every (segment, cell) of the
// realization, written over its segments' histograms.
__global__ void __launch_bounds__(kSortThreads)
    cell_scan_kernel(const Item *__restrict__ items, unsigned *__restrict__ hist) {
    __shared__ unsigned tot[kCells];
    __shared__ unsigned s_wsum[32];
    const Item it = items[blockIdx.x];
    if (it.n_seg == 0) return;
    unsigned *h = hist + it.seg_off * kCells;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int c = tid; c < kCells; c += kSortThreads) {
        unsigned t = 0;
        for (int64_t s = 0; s < it.n_seg; ++s) t += h[s * kCells + c];
        tot[c] = t;
    }
    __syncthreads();
    unsigned v[4], sum = 0;
    for (int i = 0; i < 4; ++i) {
        v[i] = tot[tid * 4 + i];
        sum += v[i];
    }
    unsigned incl = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned x = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += x;
    }
    if (lane == 31) s_wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const unsigned w = s_wsum[lane];
        unsigned wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned x = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += x;
        }
        s_wsum[lane] = wi - w;
    }
    __syncthreads();
    unsigned run = s_wsum[warp] + incl - sum;
    for (int i = 0; i < 4; ++i) {
        tot[tid * 4 + i] = run;
        run += v[i];
    }
    __syncthreads();
    for (int c = tid; c < kCells; c += kSortThreads) {
        unsigned r = tot[c];
        for (int64_t s = 0; s < it.n_seg; ++s) {
            const unsigned t = h[s * kCells + c];
            h[s * kCells + c] = r;
            r += t;
        }
    }
}

// Segment blockIdx.x scatters its points in order (warps in turn within each
// chunk of kScatterThreads points): a stable sort.  Coordinates relative to
// the realization's first point; perm holds each sorted slot's point index
// within its realization.
__global__ void __launch_bounds__(kScatterThreads)
    seg_scatter_kernel(int dim, const Item *__restrict__ items, const Seg *__restrict__ segs,
                       const double *__restrict__ pos, int64_t total_pts,
                       const double *__restrict__ box, const unsigned *__restrict__ hist,
                       double *__restrict__ sorted, int32_t *__restrict__ perm) {
    __shared__ unsigned cur[kCells];
    __shared__ unsigned s_base[kScatterThreads];
    __shared__ double s_lo[3], s_inv[3];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const Seg sg = seg_of(segs, blockIdx.x);
    const Item it = items[sg.item];
    if (tid < 32) item_cells_warp(dim, it, box, s_lo, s_inv);
    const unsigned *src = hist + static_cast<int64_t>(blockIdx.x) * kCells;
    for (int c = tid; c < kCells; c += kScatterThreads) cur[c] = src[c];
    __syncthreads();
    const double lo[3] = {s_lo[0], s_lo[1], s_lo[2]};
    const double inv[3] = {s_inv[0], s_inv[1], s_inv[2]};
    double x0[3];
    for (int d = 0; d < 3; ++d) x0[d] = item_origin(pos, total_pts, it, d, dim);
    const double *p0 = pos + it.pt_off;
    const int64_t i1 = min(sg.begin + kSegPoints, it.n_pts);
    for (int64_t c0 = sg.begin; c0 < i1; c0 += kScatterThreads) {
        const int64_t i = c0 + tid;
        const bool valid = i < i1;
        const unsigned key = valid ? point_cell(dim, p0 + i, total_pts, lo, inv)
                                   : 0xffffffffu;
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(peers) - 1;
        const unsigned rank = __popc(peers & lanemask_lt());
        for (int w = 0; w < kScatterThreads / 32; ++w) {   // warps in order
            if (warp == w && valid && lane == leader) {
                s_base[tid] = cur[key];
                cur[key] += __popc(peers);
            }
            __syncthreads();
        }
        if (valid) {
            const int64_t dst = it.pt_off + s_base[warp * 32 + leader] + rank;
            for (int d = 0; d < dim; ++d)
                sorted[d * total_pts + dst] = p0[d * total_pts + i] - x0[d];
            perm[dst] = static_cast<int32_t>(i);
        }
        __syncthreads();
    }
}

// --------------------------------------------------------- the summation --

// Work item w of the queue: tile w / n_parts, mode stages
// [(w % n_parts) stages_per_part, + stages_per_part) of its realization.
// Ensembles run whole tiles (n_parts 1) from the cost-ordered tile list; the
// single-call path uses implicit tiles -- tile t is points
// [t tile_points, + tile_points) of realization 0 -- and splits the mode
// range over n_parts when the tiles alone cannot fill the GPU, writing FP64
// partial sums [part][point] that a second kernel adds in order.
struct BatchArgs {
    const Item *items;
    const Tile *tiles;      // null: implicit tiles of realization 0
    int64_t n_work;         // work items (tiles x parts)
    int64_t n_parts;
    int64_t stages_per_part;
    int64_t tile_points;
    unsigned int *counter;
    const unsigned char *table;
    const float *kmax;
    const double *sorted;   // sorted coordinates relative to each origin
    const int32_t *perm;
    int64_t total_pts;
    const double *scales;   // per realization, may be null (then `scale`)
    double scale;
    void *out;
    int out_f32;
    double *partial;        // n_parts > 1: FP64 partial sums [part][point]
    unsigned int *err;
};

// What a ring slot holds: stage `stage` of the `n_stages` of work item
// `work` (work < 0: no more work).
struct SlotMeta {
    int64_t work;
    int32_t stage, n_stages;
};

struct WorkItem {
    Tile tile;
    Item it;
    int64_t part, mt0, n_mt;
};

template <int W>
__device__ __forceinline__ WorkItem work_item(const BatchArgs &a, int64_t w) {
    WorkItem v;
    const int64_t tile_i = w / a.n_parts;
    v.part = w - tile_i * a.n_parts;
    v.tile = a.tiles ? a.tiles[tile_i] : Tile{0, tile_i * a.tile_points};
    v.it = a.items[v.tile.item];
    const int64_t mt_all = padded_modes(v.it.n_modes, W) / W;
    v.mt0 = min(v.part * a.stages_per_part, mt_all);
    v.n_mt = min(a.stages_per_part, mt_all - v.mt0);
    return v;
}

// Shared memory: the ring of stage slots, then per consumer warp the offsets
// of the current stage's modes (radians and turns).
template <int W, int R>
constexpr size_t stage_smem_bytes() {
    return static_cast<size_t>(R) * W * kEntryBytes +
           static_cast<size_t>(kConsumerWarps) * 2 * W * 4;
}

template <int DIM, int P, int W, int CTAS, int R>
__global__ void __launch_bounds__(kThreads, CTAS) batched_kernel(const BatchArgs a) {
    constexpr uint32_t kStageBytes = static_cast<uint32_t>(W) * kEntryBytes;
    constexpr int kChunks = W / kChunk;
    static_assert(kChunks <= 32, "one chunk maximum per lane");
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t full_bar[R];
    __shared__ __align__(8) uint64_t empty_bar[R];
    __shared__ SlotMeta meta[R];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        for (int s = 0; s < R; ++s) {
            mbar_init(&full_bar[s], 1);
            mbar_init(&empty_bar[s], kConsumerWarps);
        }
        fence_mbar_init();
    }
    __syncthreads();

    if (warp == kConsumerWarps) {
        // ------------------------------------------------------ producer --
        // Pulls work items and streams their stages into the ring, one slot
        // per stage (a slot without data for an item without modes), then
        // one "no more work" slot.  Every lane waits, lane 0 issues.
        uint64_t u = 0;   // slots filled so far
        bool ok = true;
        // waits until ring slot u % R is free (its previous use consumed)
        auto claim = [&]() -> bool {
            if (u < static_cast<uint64_t>(R)) return true;
            const uint32_t ph = static_cast<uint32_t>(((u / R) - 1) & 1);
            return __shfl_sync(0xffffffffu,
                               mbar_wait(&empty_bar[u % R], ph, a.err), 0) != 0;
        };
        for (;;) {
            int64_t w = 0;
            if (lane == 0) w = atomicAdd(a.counter, 1u);
            w = __shfl_sync(0xffffffffu, w, 0);
            if (w >= a.n_work) break;
            const WorkItem v = work_item<W>(a, w);
            const unsigned char *src = a.table + (v.it.table_off + v.mt0 * W) * kEntryBytes;
            const int64_t n_slots = max(v.n_mt, int64_t(1));
            for (int64_t st = 0; st < n_slots && ok; ++st) {
                if (!(ok = claim())) break;
                const int slot = static_cast<int>(u % R);
                if (lane == 0) {
                    meta[slot] = SlotMeta{w, static_cast<int32_t>(st),
                                          static_cast<int32_t>(v.n_mt)};
                    if (v.n_mt > 0) {
                        mbar_arrive_expect_tx(&full_bar[slot], kStageBytes);
                        bulk_copy_g2s(smem + slot * kStageBytes, src + st * kStageBytes,
                                      kStageBytes, &full_bar[slot]);
                    } else {
                        mbar_arrive_local(&full_bar[slot]);
                    }
                }
                __syncwarp();
                ++u;
            }
            if (!ok) break;
        }
        if (ok && (ok = claim())) {
            if (lane == 0) {
                meta[u % R] = SlotMeta{-1, 0, 0};
                mbar_arrive_local(&full_bar[u % R]);
            }
            __syncwarp();
            ++u;
        }
        // no bulk copy may still be landing when this warp leaves: wait for
        // the last slots it filled (at most R are outstanding)
        if (lane == 0) {
            const uint64_t first = u > static_cast<uint64_t>(R) ? u - R : 0;
            mbar_drain(full_bar, R, first, u, a.err);
        }
        __syncwarp();
        return;
    }

    // ---------------------------------------------------------- consumers --
    float *s_off = reinterpret_cast<float *>(smem + R * kStageBytes) + warp * 2 * W;
    float *s_psi = s_off + W;
    bool valid[P];
    MixedPoint<DIM> mp[P], w_origin;
    float half = 0.0f;
    double acc[P];
#pragma unroll
    for (int p = 0; p < P; ++p) {
        valid[p] = false;
        acc[p] = 0.0;
    }
    WorkItem v{};   // the current work item (read at its first stage)
    for (uint64_t u = 0;; ++u) {
        const int slot = static_cast<int>(u % R);
        const bool got = __all_sync(0xffffffffu,
                                    mbar_wait(&full_bar[slot],
                                              static_cast<uint32_t>((u / R) & 1), a.err));
        if (!got) break;
        const SlotMeta m = meta[slot];
        if (m.work < 0) break;

        if (m.stage == 0) {
            v = work_item<W>(a, m.work);
            // the warp's points (relative to the realization's origin; point
            // p of lane l is tile point (warp P + p) 32 + l, so a warp holds
            // 32 P consecutive sorted points) and the centre and half extent
            // of their bounding box
            double x[P][DIM];
            double lo[DIM], hi[DIM];
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                lo[d] = INFINITY;
                hi[d] = -INFINITY;
            }
#pragma unroll
            for (int p = 0; p < P; ++p) {
                const int64_t i = v.tile.pt_begin + (warp * P + p) * 32 + lane;
                valid[p] = i < v.it.n_pts;
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    x[p][d] = valid[p] ? a.sorted[d * a.total_pts + v.it.pt_off + i] : 0.0;
                    if (valid[p]) {
                        lo[d] = fmin(lo[d], x[p][d]);
                        hi[d] = fmax(hi[d], x[p][d]);
                    }
                }
            }
            double xw[DIM];
            half = 0.0f;
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                for (int o = 16; o > 0; o >>= 1) {
                    lo[d] = fmin(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
                    hi[d] = fmax(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
                }
                // a warp without points keeps the origin (results unused)
                xw[d] = lo[d] <= hi[d] ? 0.5 * (lo[d] + hi[d]) : 0.0;
                // rounded up: the fast-chunk test must not under-estimate it
                if (lo[d] <= hi[d])
                    half = fmaxf(half,
                                 __double2float_ru(0.5 * (hi[d] - lo[d]) * (1.0 + 1e-6)));
            }
            if (!(half < INFINITY)) half = INFINITY;   // NaN / inf: exact path
#pragma unroll
            for (int p = 0; p < P; ++p) {
                double xr[DIM];
#pragma unroll
                for (int d = 0; d < DIM; ++d) xr[d] = x[p][d] - xw[d];
                mp[p] = mixed_split_point<DIM>(xr);
                acc[p] = 0.0;
            }
            w_origin = mixed_split_point<DIM>(xw);
        }

        if (m.n_stages > 0) {
            // lane c holds the largest |k|_1 of the stage's chunk c
            const float kmax_lane =
                lane < kChunks
                    ? a.kmax[(v.it.table_off + (v.mt0 + m.stage) * W) / kChunk + lane]
                    : 0.0f;
            const float *e = reinterpret_cast<const float *>(smem + slot * kStageBytes);
            // the warp's phase offsets of this stage's modes
#pragma unroll 2
            for (int j = lane; j < W; j += 32) {
                const float4 qa = reinterpret_cast<const float4 *>(e + j * kEntryFloats)[1];
                const float4 qb = reinterpret_cast<const float4 *>(e + j * kEntryFloats)[2];
                const float qh[3] = {qa.x, qa.y, qa.z};
                const float ql[3] = {qb.x, qb.y, qb.z};
                // psi_W = psi0 - <q, x_W>  (mod 1)
                const float psi_w = -mixed_turns_minus<DIM>(qh, ql, w_origin, qa.w);
                s_psi[j] = psi_w;
                s_off[j] = -kTwoPiF * psi_w;
            }
            __syncwarp();
            float accf[P];
#pragma unroll
            for (int p = 0; p < P; ++p) accf[p] = 0.0f;
#pragma unroll 1
            for (int c = 0; c < kChunks; ++c) {
                const float4 *ek = reinterpret_cast<const float4 *>(e) +
                                   c * kChunk * (kEntryFloats / 4);
                if (__shfl_sync(0xffffffffu, kmax_lane, c) * half <= kFastBound) {
#pragma unroll 8
                    for (int j = c * kChunk; j < (c + 1) * kChunk;
                         ++j, ek += kEntryFloats / 4) {
                        const float4 kk = ek[0];   // k0 k1 k2 A
                        const float off = s_off[j];
#pragma unroll
                        for (int p = 0; p < P; ++p) {
                            float arg = fmaf(kk.x, mp[p].xf[0], off);
                            if (DIM > 1) arg = fmaf(kk.y, mp[p].xf[DIM > 1 ? 1 : 0], arg);
                            if (DIM > 2) arg = fmaf(kk.z, mp[p].xf[DIM > 2 ? 2 : 0], arg);
                            accf[p] = fmaf(kk.w, __cosf(arg), accf[p]);
                        }
                    }
                } else {
#pragma unroll 2
                    for (int j = c * kChunk; j < (c + 1) * kChunk;
                         ++j, ek += kEntryFloats / 4) {
                        const float amp = ek[0].w;
                        const float4 qa = ek[1];
                        const float4 qb = ek[2];
                        const float qh[3] = {qa.x, qa.y, qa.z};
                        const float ql[3] = {qb.x, qb.y, qb.z};
                        const float psi = s_psi[j];
#pragma unroll
                        for (int p = 0; p < P; ++p) {
                            const float t = mixed_turns_minus<DIM>(qh, ql, mp[p], psi);
                            accf[p] = fmaf(amp, __cosf(t * kTwoPiF), accf[p]);
                        }
                    }
                }
            }
#pragma unroll
            for (int p = 0; p < P; ++p) acc[p] += static_cast<double>(accf[p]);
        }
        // the slot (stage data, meta and this warp's offsets) is released
        __syncwarp();
        if (lane == 0) mbar_arrive_local(&empty_bar[slot]);

        if (m.stage + 1 >= m.n_stages) {
            const double scale = a.scales ? a.scales[v.tile.item] : a.scale;
#pragma unroll
            for (int p = 0; p < P; ++p) {
                if (!valid[p]) continue;
                const int64_t i = v.it.pt_off + v.tile.pt_begin + (warp * P + p) * 32 + lane;
                const int64_t o = v.it.pt_off + a.perm[i];
                if (a.n_parts > 1)
                    a.partial[v.part * a.total_pts + o] = acc[p];
                else if (a.out_f32)
                    static_cast<float *>(a.out)[o] = static_cast<float>(scale * acc[p]);
                else
                    static_cast<double *>(a.out)[o] = scale * acc[p];
            }
        }
    }
}

template <int DIM, int V>
cudaError_t launch_shape(const BatchArgs &args, cudaStream_t s, bool set_attr) {
    constexpr Shape sh = kShapes[V];
    auto kern = batched_kernel<DIM, sh.points, sh.modes, sh.ctas, sh.ring>;
    constexpr size_t smem = stage_smem_bytes<sh.modes, sh.ring>();
    if (set_attr)
        return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(smem));
    kern<<<sm_count() * sh.ctas, kThreads, smem, s>>>(args);
    return cudaGetLastError();
}

// set_attr: raise the dynamic shared memory limit of the variant's kernel
// (host-side, before the first launch and outside any stream capture)
// instead of launching it.
template <int DIM>
cudaError_t launch_batched(int variant, const BatchArgs &args, cudaStream_t s,
                           bool set_attr) {
    switch (variant) {
        case 0: return launch_shape<DIM, 0>(args, s, set_attr);
        case 1: return launch_shape<DIM, 1>(args, s, set_attr);
        case 2: return launch_shape<DIM, 2>(args, s, set_attr);
        case 3: return launch_shape<DIM, 3>(args, s, set_attr);
        case 4: return launch_shape<DIM, 4>(args, s, set_attr);
        case 5: return launch_shape<DIM, 5>(args, s, set_attr);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t dispatch_batched(int dim, int variant, const BatchArgs &args,
                             cudaStream_t s, bool set_attr) {
    switch (dim) {
        case 1: return launch_batched<1>(variant, args, s, set_attr);
        case 2: return launch_batched<2>(variant, args, s, set_attr);
        case 3: return launch_batched<3>(variant, args, s, set_attr);
        default: return cudaErrorInvalidValue;
    }
}

std::mutex g_attr_mutex;
bool g_attr_done[3][kNumShapes];

// Raises the shared memory limit of (dim, variant) once per process.
int ensure_attr(int dim, int variant) {
    std::lock_guard<std::mutex> lock(g_attr_mutex);
    if (!g_attr_done[dim - 1][variant]) {
        GST_TRY_CUDA(dispatch_batched(dim, variant, BatchArgs{}, nullptr, true));
        g_attr_done[dim - 1][variant] = true;
    }
    return GST_OK;
}

// The prologue (mode packing, point sort) of a batch whose descriptors are
// in device memory; n_seg sort segments (segs null: the one realization's).
cudaError_t run_prologue(int dim, int64_t n_items, const Item *items, int64_t n_seg,
                         const Seg *segs, int64_t total_modes, int64_t total_pts,
                         const double *cov, const double *z1, const double *z2,
                         const double *pos, int stage_modes, float *table, float *kmax,
                         double *box, unsigned *hist, double *sorted, int32_t *perm,
                         cudaStream_t s) {
    if (n_items > 0)
        pack_batch_kernel<<<static_cast<unsigned>(n_items), kPackThreads, 0, s>>>(
            dim, items, total_modes, cov, z1, z2, pos, total_pts, stage_modes, table, kmax);
    if (n_seg > 0) {
        const unsigned g = static_cast<unsigned>(n_seg);
        seg_box_kernel<<<g, 256, 0, s>>>(dim, items, segs, pos, total_pts, box);
        seg_hist_kernel<<<g, kSortThreads, 0, s>>>(dim, items, segs, pos, total_pts, box,
                                                  hist);
        cell_scan_kernel<<<static_cast<unsigned>(n_items), kSortThreads, 0, s>>>(items,
                                                                                hist);
        seg_scatter_kernel<<<g, kScatterThreads, 0, s>>>(dim, items, segs, pos, total_pts,
                                                        box, hist, sorted, perm);
    }
    return cudaGetLastError();
}

// The one realization of the single-call path.
__global__ void single_item_kernel(Item *item, int64_t n_modes, int64_t n_pts,
                                   int64_t n_seg) {
    if (threadIdx.x == 0) *item = Item{0, n_modes, 0, 0, n_pts, 0, n_seg, 0};
}

// out[i] = scale * sum_p partial[p][i], parts in order.
__global__ void add_parts_kernel(const double *__restrict__ partial, int64_t n_parts,
                                 int64_t n, void *out, int out_f32, double scale) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int64_t p = 0; p < n_parts; ++p) s += partial[p * n + i];
    if (out_f32)
        static_cast<float *>(out)[i] = static_cast<float>(scale * s);
    else
        static_cast<double *>(out)[i] = scale * s;
}

}  // namespace

// The mixed-precision summate of one unstructured point set through the
// sorted amplitude-phase path above, as a batch of one realization
// (declared in gst_common.cuh).  Scratch from the library's stream-ordered
// pool.
int summate_mixed_sorted(int dim, int64_t n_modes, int64_t n_pts, const double *cov,
                         const double *z1, const double *z2, const double *pos,
                         void *out, int out_f32, double scale, cudaStream_t s) {
    constexpr Shape sh = kShapes[kSingleShape];
    if (dim < 1 || dim > 3) return GST_ERR_UNSUPPORTED_DIM;
    if (n_modes < 0 || n_pts < 0) return GST_ERR_INVALID_ARGUMENT;
    if (n_pts == 0) return GST_OK;
    if (out == nullptr) return GST_ERR_INVALID_ARGUMENT;
    if (current_device() < 0) return GST_ERR_NO_DEVICE;
    if (n_modes == 0) {
        GST_TRY_CUDA(cudaMemsetAsync(out, 0, (out_f32 ? 4 : 8) * n_pts, s));
        return GST_OK;
    }
    if (cov == nullptr || z1 == nullptr || z2 == nullptr || pos == nullptr)
        return GST_ERR_INVALID_ARGUMENT;
    if (n_pts > 0x7fffffffLL) return GST_ERR_TOO_LARGE;
    unsigned int *err = device_error_word();
    if (err == nullptr) return GST_ERR_CUDA;
    int rc = ensure_attr(dim, kSingleShape);
    if (rc) return rc;

    const int64_t tp = tile_points(kSingleShape);
    const int64_t n_tiles = ceil_div(n_pts, tp);
    const int64_t mt_all = padded_modes(n_modes, sh.modes) / sh.modes;
    // enough work items for two per resident CTA
    const int64_t target = static_cast<int64_t>(sm_count()) * sh.ctas * 2;
    int64_t n_parts = std::max<int64_t>(1, std::min(mt_all, ceil_div(target, n_tiles)));
    const int64_t spp = ceil_div(mt_all, n_parts);
    n_parts = ceil_div(mt_all, spp);
    const int64_t n_seg = ceil_div(n_pts, kSegPoints);

    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align_up(off + bytes, 256);
        return o;
    };
    const size_t o_item = take(sizeof(Item));
    const size_t o_counter = take(sizeof(unsigned int));
    const size_t o_table = take(static_cast<size_t>(mt_all * sh.modes) * kEntryBytes);
    const size_t o_kmax = take(sizeof(float) * static_cast<size_t>(mt_all * sh.modes / kChunk));
    const size_t o_box = take(sizeof(double) * 6 * static_cast<size_t>(n_seg));
    const size_t o_hist = take(sizeof(unsigned) * kCells * static_cast<size_t>(n_seg));
    const size_t o_sorted = take(sizeof(double) * dim * static_cast<size_t>(n_pts));
    const size_t o_perm = take(sizeof(int32_t) * static_cast<size_t>(n_pts));
    const size_t o_part =
        take(n_parts > 1 ? sizeof(double) * static_cast<size_t>(n_parts * n_pts) : 0);
    StreamScratch ws;
    GST_TRY_CUDA(ws.alloc(off, s));
    unsigned char *base = static_cast<unsigned char *>(ws.ptr);
    Item *item = reinterpret_cast<Item *>(base + o_item);

    GST_TRY_CUDA(cudaMemsetAsync(base + o_counter, 0, sizeof(unsigned int), s));
    single_item_kernel<<<1, 32, 0, s>>>(item, n_modes, n_pts, n_seg);
    GST_TRY_CUDA(run_prologue(dim, 1, item, n_seg, nullptr, n_modes, n_pts, cov, z1, z2,
                              pos, sh.modes, reinterpret_cast<float *>(base + o_table),
                              reinterpret_cast<float *>(base + o_kmax),
                              reinterpret_cast<double *>(base + o_box),
                              reinterpret_cast<unsigned *>(base + o_hist),
                              reinterpret_cast<double *>(base + o_sorted),
                              reinterpret_cast<int32_t *>(base + o_perm), s));

    BatchArgs args{};
    args.items = item;
    args.tiles = nullptr;
    args.n_work = n_tiles * n_parts;
    args.n_parts = n_parts;
    args.stages_per_part = spp;
    args.tile_points = tp;
    args.counter = reinterpret_cast<unsigned int *>(base + o_counter);
    args.table = base + o_table;
    args.kmax = reinterpret_cast<const float *>(base + o_kmax);
    args.sorted = reinterpret_cast<const double *>(base + o_sorted);
    args.perm = reinterpret_cast<const int32_t *>(base + o_perm);
    args.total_pts = n_pts;
    args.scales = nullptr;
    args.scale = scale;
    args.out = out;
    args.out_f32 = out_f32;
    args.partial = n_parts > 1 ? reinterpret_cast<double *>(base + o_part) : nullptr;
    args.err = err;
    GST_TRY_CUDA(dispatch_batched(dim, kSingleShape, args, s, false));
    if (n_parts > 1) {
        add_parts_kernel<<<static_cast<unsigned>(ceil_div(n_pts, 256)), 256, 0, s>>>(
            args.partial, n_parts, n_pts, out, out_f32, scale);
        GST_TRY_CUDA(cudaGetLastError());
    }
    return GST_OK;
}

}  // namespace gst

extern "C" {

int gst_batch_variants(void) { return gst::kNumShapes; }

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
    rc = ensure_attr(dim, variant);
    if (rc) return rc;

    std::vector<unsigned char> host(l.table_off, 0);
    Item *items = reinterpret_cast<Item *>(host.data() + l.items_off);
    Tile *tiles = reinterpret_cast<Tile *>(host.data() + l.tiles_off);
    Seg *segs = reinterpret_cast<Seg *>(host.data() + l.segs_off);
    int64_t mode_off = 0, pt_off = 0, table_off = 0, nt = 0, seg_off = 0;
    const int64_t tp = tile_points(variant);
    const int w = kShapes[variant].modes;
    std::vector<std::pair<int64_t, int64_t>> order;  // (cost, tile index)
    order.reserve(static_cast<size_t>(l.n_tiles));
    for (int64_t r = 0; r < n_items; ++r) {
        const int64_t n_seg = ceil_div(point_counts[r], kSegPoints);
        items[r] = Item{mode_off, mode_counts[r], table_off, pt_off, point_counts[r],
                        seg_off, n_seg, 0};
        for (int64_t sg = 0; sg < n_seg; ++sg) segs[seg_off + sg] = Seg{r, sg * kSegPoints};
        const int64_t padded = padded_modes(mode_counts[r], w);
        for (int64_t b = 0; b < point_counts[r]; b += tp) {
            tiles[nt] = Tile{r, b};
            order.emplace_back(padded * std::min(tp, point_counts[r] - b), nt);
            ++nt;
        }
        mode_off += mode_counts[r];
        pt_off += point_counts[r];
        table_off += padded;
        seg_off += n_seg;
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
    int64_t total_modes = 0, total_pts = 0;
    for (int64_t r = 0; r < n_items; ++r) {
        total_modes += mode_counts[r];
        total_pts += point_counts[r];
    }
    if (total_pts == 0) return GST_OK;
    if (workspace == nullptr || workspace_bytes < l.total || out == nullptr ||
        pos == nullptr)
        return GST_ERR_INVALID_ARGUMENT;
    if (total_modes > 0 && (cov == nullptr || z_1 == nullptr || z_2 == nullptr))
        return GST_ERR_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(workspace) % 256 != 0) return GST_ERR_ALIGNMENT;
    if (n_items > 0x7fffffffLL) return GST_ERR_TOO_LARGE;
    if (current_device() < 0) return GST_ERR_NO_DEVICE;
    unsigned int *err = device_error_word();
    if (err == nullptr) return GST_ERR_CUDA;
    rc = ensure_attr(dim, variant);   // done by gst_batch_prepare already
    if (rc) return rc;

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned char *ws = static_cast<unsigned char *>(workspace);
    const Item *items = reinterpret_cast<const Item *>(ws + l.items_off);
    GST_TRY_CUDA(cudaMemsetAsync(ws + l.counter_off, 0, sizeof(unsigned int), s));
    GST_TRY_CUDA(run_prologue(
        dim, n_items, items, l.n_seg, reinterpret_cast<const Seg *>(ws + l.segs_off),
        total_modes, total_pts, cov, z_1, z_2, pos, kShapes[variant].modes,
        reinterpret_cast<float *>(ws + l.table_off), reinterpret_cast<float *>(ws + l.kmax_off),
        reinterpret_cast<double *>(ws + l.box_off),
        reinterpret_cast<unsigned *>(ws + l.hist_off),
        reinterpret_cast<double *>(ws + l.sorted_off),
        reinterpret_cast<int32_t *>(ws + l.perm_off), s));
    BatchArgs args{};
    args.items = items;
    args.tiles = reinterpret_cast<const Tile *>(ws + l.tiles_off);
    args.n_work = l.n_tiles;
    args.n_parts = 1;
    args.stages_per_part = INT64_MAX;
    args.tile_points = tile_points(variant);
    args.counter = reinterpret_cast<unsigned int *>(ws + l.counter_off);
    args.table = ws + l.table_off;
    args.kmax = reinterpret_cast<const float *>(ws + l.kmax_off);
    args.sorted = reinterpret_cast<const double *>(ws + l.sorted_off);
    args.perm = reinterpret_cast<const int32_t *>(ws + l.perm_off);
    args.total_pts = total_pts;
    args.scales = scales;
    args.scale = 1.0;
    args.out = out;
    args.out_f32 = out_type == GST_OUT_F32 ? 1 : 0;
    args.partial = nullptr;
    args.err = err;
    GST_TRY_CUDA(dispatch_batched(dim, variant, args, s, false));
    return GST_OK;
}

}  // extern "C"
