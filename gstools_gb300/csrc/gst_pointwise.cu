// Pointwise randomization-method summation on sm_103a.
//
// Replaces gstools_cython.field.summate / summate_incompr / summate_fourier
// (src/gstools/field/generator.py:22-24; formulas :193-199, :479-495,
// :682-689).  One kernel template covers
//
//   KIND   scalar (summate, summate_fourier) or incompressible (summate_incompr)
//   PREC   FP64 (parity anchor) or mixed (FP32 + SFU, split turn reduction
//          of phases relative to the first point)
//   POS    unstructured points (pos is (dim, n)) or structured-grid points
//          addressed through per-axis coordinate arrays (no meshgrid in HBM)
//
// Data flow per CTA:
//   * a tile of evaluation points lives in registers for the whole kernel
//     (P points per thread, coalesced loads, one pass over HBM);
//   * the mode set has been packed by a prologue kernel into a table of
//     64-byte entries (FP64 wave vector, or its split FP32 turns for the
//     mixed path; amplitudes; projector) padded with zero-amplitude modes to
//     a whole number of tiles;
//   * mode tiles stream into shared memory through double-buffered bulk (TMA)
//     copies tracked by mbarriers, and every thread reads each entry as a
//     broadcast;
//   * when there are too few point tiles to fill 152 SMs, the mode range is
//     split across blockIdx.y and a second kernel adds the FP64 partial sums in
//     a fixed order (deterministic results).
#include <algorithm>
#include <mutex>

#include "gst_common.cuh"
#include "gst_mixed.cuh"

namespace gst {
namespace {

constexpr int kEntryBytes = 64;  // one packed mode
constexpr int kStages = 2;

// kGradPos: the position adjoint of summate,
//   out[d, i] = sum_j k_jd (z2_j cos(<k_j, x_i>) - z1_j sin(<k_j, x_i>)),
// evaluated like the incompressible sum with "projector" k and amplitudes
// (z2, -z1).
enum Kind { kScalar = 0, kIncompr = 1, kGradPos = 2 };
enum Prec { kF64 = 0, kMixed = 1 };
enum PosMode { kUnstructured = 0, kStructured = 1 };

template <int PREC>
struct Tiling;
template <>
struct Tiling<kF64> {
    static constexpr int kThreads = 128;
    static constexpr int kPoints = 2;     // points per thread
    static constexpr int kTileModes = 128;
    static constexpr int kMinBlocks = 4;
};
template <>
struct Tiling<kMixed> {
    static constexpr int kThreads = 256;
    static constexpr int kPoints = 4;
    static constexpr int kTileModes = 256;
    static constexpr int kMinBlocks = 2;
};


// ---------------------------------------------------------- mode packing --
//
// FP64 scalar entry  (8 doubles): k0 k1 k2 k3 z1 z2 f -    f = weight (1)
// FP64 incompr entry (8 doubles): k0 k1 k2 z1 z2 p0 p1 p2   p = projector
// mixed entry (16 floats): qh0 qh1 qh2 a1 | ql0 ql1 ql2 a2 | p0 p1 p2 - | ...
//                          q = k / (2 pi) split as qh (12 significant bits)
//                          + ql, so qh * xh is exact in FP32; (a1, a2) =
//                          (z1, z2) rotated by <k, x0>, x0 the first point,
//                          whose coordinates the kernel subtracts from every
//                          point (gst_mixed.cuh, rotate_to_origin).
// `weight` is summate_fourier's spectrum factor: the FP64 table keeps it as a
// separate factor (applied to z1 cos + z2 sin, as the reference does); the
// mixed table folds it into z1 and z2.
//
// The FP64 path evaluates every (mode, point) pair in the reference's own
// operation order -- phase = ((k0 x0) + k1 x1) + ..., each product and sum
// rounded separately (no FMA contraction), sin/cos of the radian phase,
// acc += (z1 cos + z2 sin) -- so it tracks the reference to a few ulp even
// where phases reach 1e5 rad.

template <int KIND, int PREC>
__global__ void pack_modes_kernel(int dim, int64_t n_modes, int64_t n_padded,
                                  const double *__restrict__ cov,
                                  const double *__restrict__ z1,
                                  const double *__restrict__ z2,
                                  const double *__restrict__ weight,
                                  const double *o0, const double *o1,
                                  const double *o2, void *__restrict__ table) {
    const int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (j >= n_padded) return;
    double k[4] = {0.0, 0.0, 0.0, 0.0};
    double a1 = 0.0, a2 = 0.0, w = 0.0;
    double proj[3] = {0.0, 0.0, 0.0};
    if (j < n_modes) {
        for (int d = 0; d < dim; ++d) k[d] = cov[d * n_modes + j];
        w = weight ? weight[j] : 1.0;
        a1 = z1[j];
        a2 = z2[j];
        if (KIND == kGradPos) {
            a1 = z2[j];
            a2 = -z1[j];
            for (int d = 0; d < dim && d < 3; ++d) proj[d] = k[d];
        }
        if (KIND == kIncompr) {
            // p_c = delta_c0 - k_c k_0 / |k|^2   (generator.py:479-495)
            double k2 = 0.0;
            for (int d = 0; d < dim; ++d) k2 = __dadd_rn(k2, __dmul_rn(k[d], k[d]));
            for (int d = 0; d < dim; ++d)
                proj[d] = __dsub_rn(d == 0 ? 1.0 : 0.0,
                                    __ddiv_rn(__dmul_rn(k[d], k[0]), k2));
        }
    }
    if (PREC == kF64) {
        double *e = static_cast<double *>(table) + j * 8;
        if (KIND == kScalar) {
            for (int d = 0; d < 4; ++d) e[d] = k[d];
            // (kIncompr and kGradPos share the layout below)
            e[4] = a1;
            e[5] = a2;
            e[6] = w;
            e[7] = 0.0;
        } else {
            for (int d = 0; d < 3; ++d) e[d] = k[d];
            e[3] = a1;
            e[4] = a2;
            for (int d = 0; d < 3; ++d) e[5 + d] = proj[d];
        }
    } else {
        // amplitudes rotated to the points' origin (gst_mixed.cuh)
        double b1 = a1 * w, b2 = a2 * w;
        const double x0[3] = {origin_coord(o0), origin_coord(o1), origin_coord(o2)};
        if (j < n_modes) rotate_to_origin(k, dim, x0, b1, b2);
        mixed_pack_entry(static_cast<float *>(table) + j * 16, k, b1, b2, proj);
    }
}

// ------------------------------------------------------------- kernel --

struct PointwiseArgs {
    const unsigned char *table;  // packed modes, kTileModes-padded
    int64_t n_tiles;             // mode tiles in the table
    int64_t tiles_per_split;     // mode tiles handled by one blockIdx.y
    int64_t n_pts;
    const double *pos;           // (dim, n_pts) for unstructured points
    const double *axes;          // concatenated axis arrays (structured)
    const double *origin[3];     // mixed: coordinates of the shift origin
    int64_t axis_len[4];
    int64_t axis_off[4];
    void *out;                   // final output, or FP64 partials
    int out_f32;                 // final output element type
    int partial;                 // 1: write partial sums [split][comp][n]
    double scale;                // applied to final outputs
    unsigned int *err;
};

template <int DIM, int POS>
__device__ __forceinline__ void load_point(const PointwiseArgs &a, int64_t i,
                                           double (&x)[DIM]) {
    if (POS == kUnstructured) {
#pragma unroll
        for (int d = 0; d < DIM; ++d) x[d] = a.pos[d * a.n_pts + i];
    } else {
        int64_t rem = i;
#pragma unroll
        for (int d = DIM - 1; d >= 0; --d) {
            const int64_t len = a.axis_len[d];
            const int64_t idx = rem % len;
            rem /= len;
            x[d] = a.axes[a.axis_off[d] + idx];
        }
    }
}

template <int DIM, int KIND, int PREC, int POS>
__global__ void __launch_bounds__(Tiling<PREC>::kThreads,
                                  Tiling<PREC>::kMinBlocks)
    pointwise_kernel(const PointwiseArgs a) {
    using T = Tiling<PREC>;
    constexpr int P = T::kPoints;
    constexpr int NT = T::kThreads;
    constexpr int TILE = T::kTileModes;
    constexpr int NC = (KIND == kScalar) ? 1 : DIM;  // output components
    constexpr uint32_t kStageBytes = TILE * kEntryBytes;

    __shared__ __align__(128) unsigned char stage[kStages][kStageBytes];
    __shared__ __align__(8) uint64_t full_bar[kStages];

    const int tid = threadIdx.x;
    const int64_t tile0 = static_cast<int64_t>(blockIdx.y) * a.tiles_per_split;
    const int64_t n_tile = min(a.tiles_per_split, a.n_tiles - tile0);

    // Evaluation points of this thread (coalesced: point p of thread t is
    // base + p * NT + t).
    const int64_t base = static_cast<int64_t>(blockIdx.x) * (P * NT);
    double x[P][DIM];
    bool valid[P];
#pragma unroll
    for (int p = 0; p < P; ++p) {
        const int64_t i = base + p * NT + tid;
        valid[p] = i < a.n_pts;
        if (valid[p]) {
            load_point<DIM, POS>(a, i, x[p]);
        } else {
#pragma unroll
            for (int d = 0; d < DIM; ++d) x[p][d] = 0.0;
        }
    }

    // Mixed precision: positions relative to the origin the mode table was
    // rotated to, split once per point.
    MixedPoint<DIM> mp[P];
    if (PREC == kMixed) {
        double x0[DIM];
#pragma unroll
        for (int d = 0; d < DIM; ++d) x0[d] = origin_coord(a.origin[d]);
#pragma unroll
        for (int p = 0; p < P; ++p) {
#pragma unroll
            for (int d = 0; d < DIM; ++d) x[p][d] -= x0[d];
            mp[p] = mixed_split_point<DIM>(x[p]);
        }
    }

    double acc[P][NC];
#pragma unroll
    for (int p = 0; p < P; ++p)
#pragma unroll
        for (int c = 0; c < NC; ++c) acc[p][c] = 0.0;

    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(&full_bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
        for (int s = 0; s < kStages && s < n_tile; ++s) {
            mbar_arrive_expect_tx(&full_bar[s], kStageBytes);
            bulk_copy_g2s(stage[s], a.table + (tile0 + s) * kStageBytes,
                          kStageBytes, &full_bar[s]);
        }
    }

    for (int64_t t = 0; t < n_tile; ++t) {
        const int s = static_cast<int>(t % kStages);
        const uint32_t parity = static_cast<uint32_t>((t / kStages) & 1);
        const bool ok = mbar_wait(&full_bar[s], parity, a.err);

        if (PREC == kF64) {
            const double *e = reinterpret_cast<const double *>(stage[s]);
#pragma unroll 1
            for (int jj = 0; jj < TILE; ++jj, e += 8) {
                const double z1 = (KIND == kScalar) ? e[4] : e[3];
                const double z2 = (KIND == kScalar) ? e[5] : e[4];
#pragma unroll
                for (int p = 0; p < P; ++p) {
                    // reference order: phase += k_d * x_d, unfused
                    double ph = __dmul_rn(e[0], x[p][0]);
#pragma unroll
                    for (int d = 1; d < DIM; ++d)
                        ph = __dadd_rn(ph, __dmul_rn(e[d], x[p][d]));
                    double sn, cs;
                    sincos(ph, &sn, &cs);
                    const double amp =
                        __dadd_rn(__dmul_rn(z1, cs), __dmul_rn(z2, sn));
                    if (KIND == kScalar) {
                        acc[p][0] = __dadd_rn(acc[p][0], __dmul_rn(e[6], amp));
                    } else {
#pragma unroll
                        for (int c = 0; c < NC; ++c)
                            acc[p][c] =
                                __dadd_rn(acc[p][c], __dmul_rn(e[5 + c], amp));
                    }
                }
            }
        } else {
            float accf[P][NC];
#pragma unroll
            for (int p = 0; p < P; ++p)
#pragma unroll
                for (int c = 0; c < NC; ++c) accf[p][c] = 0.0f;
            const float4 *e = reinterpret_cast<const float4 *>(stage[s]);
#pragma unroll 2
            for (int jj = 0; jj < TILE; ++jj, e += 4) {
                const float4 qa = e[0];  // qh0 qh1 qh2 z1
                const float4 qb = e[1];  // ql0 ql1 ql2 z2
                const float qh[3] = {qa.x, qa.y, qa.z};
                const float ql[3] = {qb.x, qb.y, qb.z};
                float4 pr = make_float4(0.f, 0.f, 0.f, 0.f);
                if (KIND != kScalar) pr = e[2];
                const float prj[3] = {pr.x, pr.y, pr.z};
#pragma unroll
                for (int p = 0; p < P; ++p) {
                    float sn, cs;
                    mixed_sincos<DIM>(qh, ql, mp[p], &sn, &cs);
                    if (KIND == kScalar) {
                        accf[p][0] = fmaf(qa.w, cs, fmaf(qb.w, sn, accf[p][0]));
                    } else {
                        const float amp = fmaf(qa.w, cs, qb.w * sn);
#pragma unroll
                        for (int c = 0; c < NC; ++c)
                            accf[p][c] = fmaf(prj[c], amp, accf[p][c]);
                    }
                }
            }
#pragma unroll
            for (int p = 0; p < P; ++p)
#pragma unroll
                for (int c = 0; c < NC; ++c)
                    acc[p][c] += static_cast<double>(accf[p][c]);
        }

        // Stage s fully consumed by every thread; agree on wait failures.
        // On a failure, tiles t .. t + kStages - 1 may still be landing in
        // shared memory: drain them before the CTA exits.
        if (__syncthreads_or(!ok)) {
            if (tid == 0)
                mbar_drain(full_bar, kStages, static_cast<uint64_t>(t),
                           static_cast<uint64_t>(min(t + kStages, n_tile)), a.err);
            break;
        }
        if (tid == 0 && t + kStages < n_tile) {
            mbar_arrive_expect_tx(&full_bar[s], kStageBytes);
            bulk_copy_g2s(stage[s], a.table + (tile0 + t + kStages) * kStageBytes,
                          kStageBytes, &full_bar[s]);
        }
    }

#pragma unroll
    for (int p = 0; p < P; ++p) {
        if (!valid[p]) continue;
        const int64_t i = base + p * NT + tid;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            if (a.partial) {
                double *w = static_cast<double *>(a.out);
                w[(static_cast<int64_t>(blockIdx.y) * NC + c) * a.n_pts + i] =
                    acc[p][c];
            } else if (a.out_f32) {
                static_cast<float *>(a.out)[c * a.n_pts + i] =
                    static_cast<float>(a.scale * acc[p][c]);
            } else {
                static_cast<double *>(a.out)[c * a.n_pts + i] =
                    a.scale * acc[p][c];
            }
        }
    }
}

// Adds the split-mode partial sums in split order (deterministic).
__global__ void reduce_partials_kernel(const double *__restrict__ partial,
                                       int64_t n_split, int64_t n_values,
                                       void *out, int out_f32, double scale) {
    const int64_t v = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (v >= n_values) return;
    double s = 0.0;
    for (int64_t k = 0; k < n_split; ++k) s += partial[k * n_values + v];
    if (out_f32)
        static_cast<float *>(out)[v] = static_cast<float>(scale * s);
    else
        static_cast<double *>(out)[v] = scale * s;
}

// --------------------------------------------------------------- host --

struct Request {
    int kind;            // Kind
    int prec;            // Prec
    int pos_mode;        // PosMode
    int dim;
    int64_t n_modes;
    int64_t n_pts;
    const double *cov;
    const double *z1;
    const double *z2;
    const double *weight;  // spectrum factor (summate_fourier) or null
    const double *pos;
    const double *axes;
    int64_t axis_len[4];
    void *out;
    int out_f32;
    double scale;
    cudaStream_t stream;
};

template <int DIM, int KIND, int PREC, int POS>
cudaError_t launch_main(dim3 grid, const PointwiseArgs &args, cudaStream_t s) {
    pointwise_kernel<DIM, KIND, PREC, POS>
        <<<grid, Tiling<PREC>::kThreads, 0, s>>>(args);
    return cudaGetLastError();
}

template <int KIND, int PREC, int POS>
cudaError_t dispatch_dim(int dim, dim3 grid, const PointwiseArgs &args,
                         cudaStream_t s) {
    if (KIND == kGradPos) {
        switch (dim) {
            case 1: return launch_main<1, KIND, PREC, POS>(grid, args, s);
            case 2: return launch_main<2, KIND, PREC, POS>(grid, args, s);
            case 3: return launch_main<3, KIND, PREC, POS>(grid, args, s);
            default: return cudaErrorInvalidValue;
        }
    }
    if (KIND == kIncompr) {
        switch (dim) {
            case 2: return launch_main<2, KIND, PREC, POS>(grid, args, s);
            case 3: return launch_main<3, KIND, PREC, POS>(grid, args, s);
            default: return cudaErrorInvalidValue;
        }
    }
    switch (dim) {
        case 1: return launch_main<1, KIND, PREC, POS>(grid, args, s);
        case 2: return launch_main<2, KIND, PREC, POS>(grid, args, s);
        case 3: return launch_main<3, KIND, PREC, POS>(grid, args, s);
        case 4:
            if (PREC == kF64) return launch_main<4, KIND, kF64, POS>(grid, args, s);
            return cudaErrorInvalidValue;
        default: return cudaErrorInvalidValue;
    }
}

template <int KIND, int PREC>
cudaError_t dispatch(int pos_mode, int dim, dim3 grid, const PointwiseArgs &args,
                     cudaStream_t s) {
    if (pos_mode == kStructured)
        return dispatch_dim<KIND, PREC, kStructured>(dim, grid, args, s);
    return dispatch_dim<KIND, PREC, kUnstructured>(dim, grid, args, s);
}

// Device addresses of the coordinates of the mixed paths' shift origin: the
// first point (unstructured) or the first value of each axis (structured).
void origin_ptrs(const Request &r, const double *(&o)[3]) {
    int64_t off = 0;
    for (int d = 0; d < 3; ++d) {
        o[d] = nullptr;
        if (d >= r.dim || r.n_pts == 0) continue;
        if (r.pos_mode == kUnstructured) {
            o[d] = r.pos + d * r.n_pts;
        } else {
            o[d] = r.axes + off;
            off += r.axis_len[d];
        }
    }
}

template <int KIND, int PREC>
void pack(const Request &r, int64_t n_padded, void *table) {
    // small blocks: the mixed entries' FP64 origin rotation is FP64-pipe
    // work, spread over many SMs (256-thread blocks put 1000 modes on 4 SMs)
    const int threads = 64;
    const int64_t blocks = ceil_div(n_padded, threads);
    const double *o[3];
    origin_ptrs(r, o);
    pack_modes_kernel<KIND, PREC><<<static_cast<unsigned>(blocks), threads, 0,
                                    r.stream>>>(r.dim, r.n_modes, n_padded,
                                                r.cov, r.z1, r.z2, r.weight,
                                                o[0], o[1], o[2], table);
}

int run(const Request &r) {
    const int nc = (r.kind == kScalar) ? 1 : r.dim;
    if (r.kind == kIncompr) {
        if (r.dim < 2 || r.dim > 3) return GST_ERR_UNSUPPORTED_DIM;
    } else if (r.kind == kGradPos) {
        if (r.dim < 1 || r.dim > 3) return GST_ERR_UNSUPPORTED_DIM;
    } else {
        const int max_dim = (r.prec == kF64) ? 4 : 3;
        if (r.dim < 1 || r.dim > max_dim) return GST_ERR_UNSUPPORTED_DIM;
    }
    if (r.n_modes < 0 || r.n_pts < 0) return GST_ERR_INVALID_ARGUMENT;
    if (r.pos_mode == kStructured) {
        int64_t total = 1;
        for (int d = 0; d < r.dim; ++d) {
            if (r.axis_len[d] < 0) return GST_ERR_INVALID_ARGUMENT;
            total *= r.axis_len[d];
        }
        if (total != r.n_pts) return GST_ERR_INVALID_ARGUMENT;
    }
    if (r.n_pts == 0) return GST_OK;
    if (r.out == nullptr) return GST_ERR_INVALID_ARGUMENT;
    if (gst::current_device() < 0) return GST_ERR_NO_DEVICE;
    const size_t elem = r.out_f32 ? sizeof(float) : sizeof(double);
    if (r.n_modes == 0) {
        GST_TRY_CUDA(cudaMemsetAsync(r.out, 0, elem * nc * r.n_pts, r.stream));
        return GST_OK;
    }
    if (r.cov == nullptr || r.z1 == nullptr || r.z2 == nullptr)
        return GST_ERR_INVALID_ARGUMENT;
    if (r.pos_mode == kUnstructured ? r.pos == nullptr : r.axes == nullptr)
        return GST_ERR_INVALID_ARGUMENT;

    const int threads = (r.prec == kF64) ? Tiling<kF64>::kThreads
                                         : Tiling<kMixed>::kThreads;
    const int points = (r.prec == kF64) ? Tiling<kF64>::kPoints
                                        : Tiling<kMixed>::kPoints;
    const int tile_modes = (r.prec == kF64) ? Tiling<kF64>::kTileModes
                                            : Tiling<kMixed>::kTileModes;
    const int min_blocks = (r.prec == kF64) ? Tiling<kF64>::kMinBlocks
                                            : Tiling<kMixed>::kMinBlocks;

    const int64_t n_tiles = ceil_div(r.n_modes, tile_modes);
    const int64_t n_padded = n_tiles * tile_modes;
    const int64_t pts_per_cta = static_cast<int64_t>(threads) * points;
    const int64_t n_pt_tiles = ceil_div(r.n_pts, pts_per_cta);
    if (n_pt_tiles > 0x7fffffffLL) return GST_ERR_TOO_LARGE;

    // Split the mode range when the point tiles alone cannot fill the GPU
    // (two waves of resident CTAs on every SM).
    const int64_t target = static_cast<int64_t>(gst::sm_count()) * min_blocks * 2;
    int64_t n_split = std::min<int64_t>(n_tiles, ceil_div(target, n_pt_tiles));
    n_split = std::max<int64_t>(n_split, 1);
    const int64_t tiles_per_split = ceil_div(n_tiles, n_split);
    n_split = ceil_div(n_tiles, tiles_per_split);
    if (n_split > 65535) return GST_ERR_TOO_LARGE;

    const size_t table_bytes = static_cast<size_t>(n_padded) * kEntryBytes;
    const size_t part_off = align_up(table_bytes, 256);
    const size_t part_bytes =
        n_split > 1 ? sizeof(double) * n_split * nc * r.n_pts : 0;

    unsigned int *err = gst::device_error_word();
    if (err == nullptr) return GST_ERR_CUDA;

    StreamScratch ws;
    GST_TRY_CUDA(ws.alloc(part_off + part_bytes, r.stream));
    unsigned char *table = static_cast<unsigned char *>(ws.ptr);
    double *partial =
        n_split > 1 ? reinterpret_cast<double *>(table + part_off) : nullptr;

    if (r.kind == kScalar) {
        if (r.prec == kF64) pack<kScalar, kF64>(r, n_padded, table);
        else pack<kScalar, kMixed>(r, n_padded, table);
    } else if (r.kind == kIncompr) {
        if (r.prec == kF64) pack<kIncompr, kF64>(r, n_padded, table);
        else pack<kIncompr, kMixed>(r, n_padded, table);
    } else {
        if (r.prec == kF64) pack<kGradPos, kF64>(r, n_padded, table);
        else pack<kGradPos, kMixed>(r, n_padded, table);
    }
    GST_TRY_CUDA(cudaGetLastError());

    PointwiseArgs args{};
    args.table = table;
    args.n_tiles = n_tiles;
    args.tiles_per_split = tiles_per_split;
    args.n_pts = r.n_pts;
    args.pos = r.pos;
    args.axes = r.axes;
    origin_ptrs(r, args.origin);
    int64_t off = 0;
    for (int d = 0; d < 4; ++d) {
        args.axis_len[d] = d < r.dim ? r.axis_len[d] : 1;
        args.axis_off[d] = off;
        if (d < r.dim) off += r.axis_len[d];
    }
    args.out = n_split > 1 ? static_cast<void *>(partial) : r.out;
    args.out_f32 = r.out_f32;
    args.partial = n_split > 1 ? 1 : 0;
    args.scale = r.scale;
    args.err = err;

    const dim3 grid(static_cast<unsigned>(n_pt_tiles),
                    static_cast<unsigned>(n_split));
    cudaError_t e;
    if (r.kind == kScalar)
        e = (r.prec == kF64) ? dispatch<kScalar, kF64>(r.pos_mode, r.dim, grid, args, r.stream)
                             : dispatch<kScalar, kMixed>(r.pos_mode, r.dim, grid, args, r.stream);
    else if (r.kind == kIncompr)
        e = (r.prec == kF64) ? dispatch<kIncompr, kF64>(r.pos_mode, r.dim, grid, args, r.stream)
                             : dispatch<kIncompr, kMixed>(r.pos_mode, r.dim, grid, args, r.stream);
    else
        e = (r.prec == kF64) ? dispatch<kGradPos, kF64>(r.pos_mode, r.dim, grid, args, r.stream)
                             : dispatch<kGradPos, kMixed>(r.pos_mode, r.dim, grid, args, r.stream);
    GST_TRY_CUDA(e);

    if (n_split > 1) {
        const int64_t n_values = nc * r.n_pts;
        const int rt = 256;
        reduce_partials_kernel<<<static_cast<unsigned>(ceil_div(n_values, rt)), rt,
                                 0, r.stream>>>(partial, n_split, n_values, r.out,
                                                r.out_f32, r.scale);
        GST_TRY_CUDA(cudaGetLastError());
    }
    return GST_OK;
}

Request make_request(int kind, int prec, int dim, int64_t n_modes, int64_t n_pts,
                     const double *cov, const double *z1, const double *z2,
                     const double *pos, void *out, int out_type, void *stream) {
    Request r{};
    r.kind = kind;
    r.prec = prec;
    r.pos_mode = kUnstructured;
    r.dim = dim;
    r.n_modes = n_modes;
    r.n_pts = n_pts;
    r.cov = cov;
    r.z1 = z1;
    r.z2 = z2;
    r.pos = pos;
    r.out = out;
    r.out_f32 = out_type == GST_OUT_F32 ? 1 : 0;
    r.scale = 1.0;
    r.stream = static_cast<cudaStream_t>(stream);
    return r;
}

int set_grid(Request &r, const int64_t *axis_len, const double *axes) {
    if (axis_len == nullptr) return GST_ERR_INVALID_ARGUMENT;
    if (r.dim < 1 || r.dim > 4) return GST_ERR_UNSUPPORTED_DIM;
    int64_t total = 1;
    for (int d = 0; d < r.dim; ++d) {
        if (axis_len[d] < 0) return GST_ERR_INVALID_ARGUMENT;
        r.axis_len[d] = axis_len[d];
        total *= axis_len[d];
    }
    r.pos_mode = kStructured;
    r.axes = axes;
    r.n_pts = total;
    return GST_OK;
}

bool valid_out_type(int t) { return t == GST_OUT_F64 || t == GST_OUT_F32; }

}  // namespace
}  // namespace gst

extern "C" {

int gst_summate_f64(int dim, int64_t n_modes, int64_t n_pts,
                    const double *cov_samples, const double *z_1,
                    const double *z_2, const double *pos, double *out,
                    void *stream) {
    auto r = gst::make_request(gst::kScalar, gst::kF64, dim, n_modes, n_pts,
                               cov_samples, z_1, z_2, pos, out, GST_OUT_F64,
                               stream);
    return gst::run(r);
}

int gst_summate_incompr_f64(int dim, int64_t n_modes, int64_t n_pts,
                            const double *cov_samples, const double *z_1,
                            const double *z_2, const double *pos, double *out,
                            void *stream) {
    auto r = gst::make_request(gst::kIncompr, gst::kF64, dim, n_modes, n_pts,
                               cov_samples, z_1, z_2, pos, out, GST_OUT_F64,
                               stream);
    return gst::run(r);
}

int gst_summate_fourier_f64(int dim, int64_t n_modes, int64_t n_pts,
                            const double *spectrum_factor, const double *modes,
                            const double *z_1, const double *z_2,
                            const double *pos, double *out, void *stream) {
    if (spectrum_factor == nullptr && n_modes > 0 && n_pts > 0)
        return GST_ERR_INVALID_ARGUMENT;
    auto r = gst::make_request(gst::kScalar, gst::kF64, dim, n_modes, n_pts,
                               modes, z_1, z_2, pos, out, GST_OUT_F64, stream);
    r.weight = spectrum_factor;
    return gst::run(r);
}

int gst_summate_vjp_pos_f64(int dim, int64_t n_modes, int64_t n_pts,
                            const double *cov_samples, const double *z_1,
                            const double *z_2, const double *pos, double *out,
                            void *stream) {
    auto r = gst::make_request(gst::kGradPos, gst::kF64, dim, n_modes, n_pts,
                               cov_samples, z_1, z_2, pos, out, GST_OUT_F64,
                               stream);
    return gst::run(r);
}

int gst_summate_vjp_pos_mixed(int dim, int64_t n_modes, int64_t n_pts,
                              const double *cov_samples, const double *z_1,
                              const double *z_2, const double *pos, double *out,
                              void *stream) {
    auto r = gst::make_request(gst::kGradPos, gst::kMixed, dim, n_modes, n_pts,
                               cov_samples, z_1, z_2, pos, out, GST_OUT_F64,
                               stream);
    return gst::run(r);
}

int gst_summate_mixed(int dim, int64_t n_modes, int64_t n_pts,
                      const double *cov_samples, const double *z_1,
                      const double *z_2, const double *pos, void *out,
                      int out_type, void *stream) {
    if (!gst::valid_out_type(out_type)) return GST_ERR_INVALID_ARGUMENT;
    // Large sums take the sorted amplitude-phase path (gst_batched.cu): its
    // prologue (mode and point sorts, ~0.15 ms at 1e5 points) pays off from
    // about 4e8 mode-points over 2e5 points on; smaller ones, and mode sets
    // beyond what its one-CTA mode sort handles quickly, run the pointwise
    // kernel here.
    const double work = static_cast<double>(n_modes) * static_cast<double>(n_pts);
    if (n_modes > 0 && n_pts > 0 && n_modes <= gst::kSortedMaxModes &&
        (work >= gst::kSortedMinWork ||
         (dim >= 2 && work >= gst::kSortedMinWorkPts && n_pts >= gst::kSortedMinPts)))
        return gst::summate_mixed_sorted(dim, n_modes, n_pts, cov_samples, z_1, z_2, pos,
                                         out, out_type == GST_OUT_F32 ? 1 : 0, 1.0,
                                         static_cast<cudaStream_t>(stream));
    auto r = gst::make_request(gst::kScalar, gst::kMixed, dim, n_modes, n_pts,
                               cov_samples, z_1, z_2, pos, out, out_type, stream);
    return gst::run(r);
}

int gst_summate_incompr_mixed(int dim, int64_t n_modes, int64_t n_pts,
                              const double *cov_samples, const double *z_1,
                              const double *z_2, const double *pos, void *out,
                              int out_type, void *stream) {
    if (!gst::valid_out_type(out_type)) return GST_ERR_INVALID_ARGUMENT;
    auto r = gst::make_request(gst::kIncompr, gst::kMixed, dim, n_modes, n_pts,
                               cov_samples, z_1, z_2, pos, out, out_type, stream);
    return gst::run(r);
}

int gst_summate_grid_f64(int dim, int64_t n_modes, const int64_t *axis_len,
                         const double *axes, const double *cov_samples,
                         const double *z_1, const double *z_2, double *out,
                         void *stream) {
    auto r = gst::make_request(gst::kScalar, gst::kF64, dim, n_modes, 0,
                               cov_samples, z_1, z_2, nullptr, out, GST_OUT_F64,
                               stream);
    const int rc = gst::set_grid(r, axis_len, axes);
    return rc ? rc : gst::run(r);
}

int gst_summate_grid_mixed(int dim, int64_t n_modes, const int64_t *axis_len,
                           const double *axes, const double *cov_samples,
                           const double *z_1, const double *z_2, void *out,
                           int out_type, double scale, void *stream) {
    if (!gst::valid_out_type(out_type)) return GST_ERR_INVALID_ARGUMENT;
    auto r = gst::make_request(gst::kScalar, gst::kMixed, dim, n_modes, 0,
                               cov_samples, z_1, z_2, nullptr, out, out_type,
                               stream);
    r.scale = scale;
    const int rc = gst::set_grid(r, axis_len, axes);
    return rc ? rc : gst::run(r);
}

int gst_summate_incompr_grid_f64(int dim, int64_t n_modes,
                                 const int64_t *axis_len, const double *axes,
                                 const double *cov_samples, const double *z_1,
                                 const double *z_2, double *out, void *stream) {
    auto r = gst::make_request(gst::kIncompr, gst::kF64, dim, n_modes, 0,
                               cov_samples, z_1, z_2, nullptr, out, GST_OUT_F64,
                               stream);
    const int rc = gst::set_grid(r, axis_len, axes);
    return rc ? rc : gst::run(r);
}

int gst_summate_incompr_grid_mixed(int dim, int64_t n_modes,
                                   const int64_t *axis_len, const double *axes,
                                   const double *cov_samples, const double *z_1,
                                   const double *z_2, void *out, int out_type,
                                   double scale, void *stream) {
    if (!gst::valid_out_type(out_type)) return GST_ERR_INVALID_ARGUMENT;
    auto r = gst::make_request(gst::kIncompr, gst::kMixed, dim, n_modes, 0,
                               cov_samples, z_1, z_2, nullptr, out, out_type,
                               stream);
    r.scale = scale;
    const int rc = gst::set_grid(r, axis_len, axes);
    return rc ? rc : gst::run(r);
}

}  // extern "C"

// ===================================================================
// Allocation-free FP64 summate.
//
// Some callers cannot let a library allocate device memory: hosts that
// reserve the GPU's memory for their own pool at start-up and forbid other
// allocations, and latency-critical loops that cannot pay for an
// allocator call.  gst_summate_f64_noalloc serves them with the FP64
// pointwise kernel above, taking its scratch (the packed mode table and the
// split-mode partial sums) from a fixed array in device memory instead of
// the stream-ordered allocator.
//
// * The array is a file-scope __device__ object of kNoAllocScratchBytes
//   (5 MiB): every GPU that loads this library holds it until the process
//   exits.  Limits: at most kNoAllocMaxModes modes; the mode range is split
//   across CTAs only as far as the partial sums fit in the remaining 4 MiB.
// * Host code cannot use the array's name as a device address.  The first
//   call on each device (with that device current) looks the address up
//   with cudaGetSymbolAddress and caches it; make that first call before
//   any stream capture (a first call on a capturing stream is refused with
//   GST_ERR_INVALID_ARGUMENT).
// * Every call shares the one array, which keeps the previous call's
//   contents.  Nothing in it has to start at zero (each call overwrites the
//   table and every partial sum it reads), but calls that overlap on the
//   GPU (different streams, or different host threads without ordering)
//   race on it and must be serialised by the caller.
// ===================================================================
namespace gst {
namespace {

constexpr int64_t kNoAllocMaxModes = 16384;
constexpr size_t kNoAllocTableBytes =
    static_cast<size_t>(kNoAllocMaxModes) * kEntryBytes;  // 1 MiB
constexpr size_t kNoAllocPartialBytes = size_t(4) << 20;    // 4 MiB
constexpr size_t kNoAllocScratchBytes = kNoAllocTableBytes + kNoAllocPartialBytes;

static __device__ __align__(256) unsigned char
    g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
unsigned char *g_noalloc_ptr[kNoAllocMaxDevices];

// Device address of g_noalloc_scratch on the current device (looked up
// once per device), or an error status.
int noalloc_scratch(unsigned char **ptr) {
    const int dev = current_device();
    if (dev < 0 || dev >= kNoAllocMaxDevices) return GST_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (g_noalloc_ptr[dev] == nullptr) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            note_cuda_error(e);
            return GST_ERR_CUDA;
        }
        // the other per-device lookups of this entry point, done here so
        // that a call under capture never performs them
        if (device_error_word() == nullptr) return GST_ERR_CUDA;
        (void)sm_count();
        g_noalloc_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *ptr = g_noalloc_ptr[dev];
    return GST_OK;
}

// Whether the first-call set-up (scratch address, error word, SM count) of
// the current device is done.
bool noalloc_ready() {
    const int dev = current_device();
    if (dev < 0 || dev >= kNoAllocMaxDevices) return false;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    return g_noalloc_ptr[dev] != nullptr;
}

int run_noalloc_f64(const Request &r) {
    if (r.dim < 1 || r.dim > 4) return GST_ERR_UNSUPPORTED_DIM;
    if (r.n_modes < 0 || r.n_pts < 0) return GST_ERR_INVALID_ARGUMENT;
    if (r.n_modes > kNoAllocMaxModes) return GST_ERR_TOO_LARGE;
    if (r.n_pts == 0) return GST_OK;
    if (r.out == nullptr) return GST_ERR_INVALID_ARGUMENT;
    if (current_device() < 0) return GST_ERR_NO_DEVICE;
    if (r.n_modes == 0) {
        GST_TRY_CUDA(cudaMemsetAsync(r.out, 0, sizeof(double) * r.n_pts, r.stream));
        return GST_OK;
    }
    if (r.cov == nullptr || r.z1 == nullptr || r.z2 == nullptr || r.pos == nullptr)
        return GST_ERR_INVALID_ARGUMENT;

    // The first call on a device looks up addresses (cudaGetSymbolAddress)
    // and the SM count; inside a stream capture that set-up is refused with
    // a clear status instead of failing in the middle of the capture.
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    GST_TRY_CUDA(cudaStreamIsCapturing(r.stream, &capture));
    if (capture != cudaStreamCaptureStatusNone && !noalloc_ready())
        return GST_ERR_INVALID_ARGUMENT;

    unsigned char *scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    unsigned int *err = device_error_word();
    if (err == nullptr) return GST_ERR_CUDA;

    using T = Tiling<kF64>;
    const int64_t n_tiles = ceil_div(r.n_modes, T::kTileModes);
    const int64_t n_padded = n_tiles * T::kTileModes;
    const int64_t pts_per_cta = static_cast<int64_t>(T::kThreads) * T::kPoints;
    const int64_t n_pt_tiles = ceil_div(r.n_pts, pts_per_cta);
    if (n_pt_tiles > 0x7fffffffLL) return GST_ERR_TOO_LARGE;

    const int64_t target = static_cast<int64_t>(sm_count()) * T::kMinBlocks * 2;
    int64_t n_split = std::min<int64_t>(n_tiles, ceil_div(target, n_pt_tiles));
    // the partial sums must fit in the fixed partial region
    const int64_t fit = static_cast<int64_t>(kNoAllocPartialBytes /
                                             (sizeof(double) * r.n_pts));
    n_split = std::max<int64_t>(1, std::min(n_split, fit));
    const int64_t tiles_per_split = ceil_div(n_tiles, n_split);
    n_split = ceil_div(n_tiles, tiles_per_split);

    unsigned char *table = scratch;
    double *partial = reinterpret_cast<double *>(scratch + kNoAllocTableBytes);
    pack<kScalar, kF64>(r, n_padded, table);
    GST_TRY_CUDA(cudaGetLastError());

    PointwiseArgs args{};
    args.table = table;
    args.n_tiles = n_tiles;
    args.tiles_per_split = tiles_per_split;
    args.n_pts = r.n_pts;
    args.pos = r.pos;
    for (int d = 0; d < 4; ++d) {
        args.axis_len[d] = 1;
        args.axis_off[d] = 0;
    }
    args.out = n_split > 1 ? static_cast<void *>(partial) : r.out;
    args.out_f32 = 0;
    args.partial = n_split > 1 ? 1 : 0;
    args.scale = 1.0;
    args.err = err;
    const dim3 grid(static_cast<unsigned>(n_pt_tiles), static_cast<unsigned>(n_split));
    GST_TRY_CUDA((dispatch<kScalar, kF64>(kUnstructured, r.dim, grid, args, r.stream)));
    if (n_split > 1) {
        const int rt = 256;
        reduce_partials_kernel<<<static_cast<unsigned>(ceil_div(r.n_pts, rt)), rt, 0,
                                 r.stream>>>(partial, n_split, r.n_pts, r.out, 0, 1.0);
        GST_TRY_CUDA(cudaGetLastError());
    }
    return GST_OK;
}

}  // namespace
}  // namespace gst

extern "C" int gst_summate_f64_noalloc(int dim, int64_t n_modes, int64_t n_pts,
                                       const double *cov_samples,
                                       const double *z_1, const double *z_2,
                                       const double *pos, double *out,
                                       void *stream) {
    auto r = gst::make_request(gst::kScalar, gst::kF64, dim, n_modes, n_pts,
                               cov_samples, z_1, z_2, pos, out, GST_OUT_F64,
                               stream);
    return gst::run_noalloc_f64(r);
}
