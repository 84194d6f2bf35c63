// Separable structured-grid summation on the sm_103a tensor cores (tcgen05).
//
// On a structured grid the phase separates per axis, exp(i<k, x>) =
// Ex[ix] Ey[iy] Ez[iz], so with w_j = z1_j - i z2_j the reference sum
// (src/gstools/field/generator.py:193-199 on the meshgrid of
// src/gstools/tools/geometric.py:340-356) becomes
//
//     F[(ix, iy), iz] = Re sum_j P_j(ix, iy) Q_j(iz),
//     P_j = w_j Ex[ix, j] Ey[iy, j],   Q_j = Ez[iz, j]
//
// a real GEMM with K = 2N (real and imaginary parts): rows are (x, y) pairs
// (operand A = [Re P, -Im P], generated on the fly), columns are z points
// (operand B = [Re Q, Im Q], a precomputed table).  A linear isometrize map
// M is folded into the wave vectors by the caller (<k, M x> = <M^T k, x>).
// A 2-D grid is the same with a dummy y axis of length 1 (Ey = 1).
//
// Precision: the per-axis tables come from an exact turn reduction of
// k x / (2 pi) and an FP32 sincospi of the reduced angle; every operand is
// split into hi + lo parts of the operand format (FP16 by default, amplitudes
// scaled by a power of two into FP16 range; TF32 selectable) and the GEMM
// runs as Ah Bh + Ah Bl + Al Bh.  The tensor core's FP32 accumulation is not
// round-to-nearest over long K, so the modes are processed in chunks (128
// modes with FP16 operands, 32 with TF32): each chunk accumulates from zero
// in tensor memory and is then added into FP32 registers of the epilogue
// threads.  Two accumulators alternate, so the tensor cores fill one while
// the other is drained.
//
// Kernel structure: a cluster of two CTAs (tcgen05 cta_group::2) per output
// tile of 256 (x, y) rows (128 per CTA) by NT z points (NT = 128, 192 or
// 256, picked per grid), M = 256, N = NT; 576 threads per CTA:
//   warp 0      bulk-copy producer: per stage its CTA's half (NT / 2 points)
//               of the pre-split Ez image (already in the UMMA canonical
//               K-major layout) and the stage's w*Ex and Ey table slices,
//               into a ring of >= 3 shared-memory slots;
//   warp 1      leader CTA: allocates 512 TMEM columns (two accumulators)
//               and issues tcgen05.mma from one lane, 3 MMAs per K-step;
//               peer CTA: relays its generators' and drains' arrivals to the
//               leader's barriers;
//   warps 2-17  generate A = w Ex Ey (complex product, hi + lo split) for
//               the CTA's 128 rows, drain finished chunk accumulators into
//               registers (tcgen05.ld), and store the tile (float32 through
//               shared memory as whole row runs).
// Tiles of a last partial wave are split over their modes in two parts that
// add into a zeroed output.  Every mbarrier wait is bounded; a timeout is
// recorded in the device error word and the CTAs still free their tensor
// memory.
#include <cuda_fp16.h>

#include <algorithm>
#include <atomic>
#include <cstring>

#include "gst_common.cuh"
#include "gst_mixed.cuh"

namespace gst {
namespace {

constexpr int kThreads = 576;
constexpr int kGenThreads = 512;      // warps 2-17
constexpr int kCtaRows = 128;         // (x, y) rows held by each CTA
constexpr int kBlockBytes = 128 * 32;  // A: 128 rows x 32 bytes of K (one K-step)
constexpr uint32_t kTmemCols = 512;  // two accumulators of up to 256 columns

// z points per pair tile (the MMA's N): 256, 192 or 128, picked per grid so
// that the padded z extent is smallest (ties to the wider tile).  Each CTA of
// a pair holds NT / 2 rows of B; each generator warp drains and stores a
// quarter (NT / 4 columns) of its accumulator rows.
__host__ __device__ constexpr int b_block_bytes(int nt) { return nt / 2 * 32; }

// Operand kinds of the split GEMM.  Both carry 10 explicit mantissa bits, so
// the three-product split (hi*hi + hi*lo + lo*hi) has the same precision;
// FP16 products run at twice the TF32 rate and move half the bytes, but need
// the amplitudes normalised into FP16 range (a power of two taken out of
// w = z1 - i z2 and put back in the epilogue).
enum OperandKind { kOpTf32 = GST_TC_TF32, kOpF16 = GST_TC_F16 };

// Modes per pipeline stage: 32 (FP16) / 16 (TF32), 4 MMA K-steps per
// operand format, so a stage is about 70 KB of shared memory either way (a
// 3-deep ring); measured on the 256^3 workload, 32-mode FP16 stages contract
// 16 % faster than 16-mode ones (half the barrier round trips per mode).
// 2-D grids (TY = 1) have A = w Ex with no y factor: the tables kernel writes
// it pre-split in the operand layout and it is bulk-copied like B, so the
// generator warps only drain and store (kACopied).
__host__ __device__ constexpr int modes_per_stage(int /*ty*/, int op) {
    return 16 * (op == kOpF16 ? 2 : 1);
}
__host__ __device__ constexpr bool a_copied(int ty) { return ty == 1; }
// Modes per MMA K-step (32 bytes of K per row: 8 TF32 or 16 FP16 reals).
__host__ __device__ constexpr int modes_per_kstep(int op) { return op == kOpF16 ? 8 : 4; }
__host__ __device__ constexpr int ksteps_for(int ty, int op) {
    return modes_per_stage(ty, op) / modes_per_kstep(op);
}
__host__ __device__ constexpr int elem_bytes(int op) { return op == kOpF16 ? 2 : 4; }
// Modes accumulated per TMEM chunk before the epilogue warps add the chunk
// into FP32 registers: 24 MMAs of K = 32 bytes per chunk with TF32 operands
// (32 modes), 48 with FP16 operands (128 modes; half the drains of 64-mode
// chunks, 4 % faster on the 256^3 workload), which keeps the tensor core's
// accumulation error near 1e-6 sigma of the field.
__host__ __device__ constexpr int chunk_modes(int op) { return op == kOpF16 ? 128 : 32; }

constexpr double kInv2Pi = 0.15915494309189533576888376337251436;

// Byte offset of element (row, k) inside one canonical K-major block of
// 8-row x 16-byte core matrices: core (row/8, k/E) sits at
// (row/8) * SBO + (k/E) * LBO with LBO = 128 B, SBO = 256 B, E = 16 bytes /
// element size.
__host__ __device__ constexpr uint32_t core_offset(uint32_t row, uint32_t k, int op) {
    return (row >> 3) * 256u + (k / (16u / elem_bytes(op))) * 128u + (row & 7u) * 16u +
           (k % (16u / elem_bytes(op))) * elem_bytes(op);
}

std::atomic<int> g_operand_kind{kOpF16};

__device__ __forceinline__ float to_tf32(float v) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
    return __uint_as_float(r);
}

// ------------------------------------------------------------ descriptors --

// tcgen05 shared-memory matrix descriptor, K-major, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);          // start
    d |= static_cast<uint64_t>((128u >> 4) & 0x3FFFu) << 16;     // LBO
    d |= static_cast<uint64_t>((256u >> 4) & 0x3FFFu) << 32;     // SBO
    d |= static_cast<uint64_t>(1u) << 46;                        // version
    return d;                                                    // swizzle 0
}

// Instruction descriptor, D = F32, A and B K-major, M = 256 (a CTA pair),
// N = NT: kind::tf32 with A = B = TF32, kind::f16 with A = B = F16.
template <int OP, int NT>
constexpr uint32_t idesc() {
    return (1u << 4)                                  // D format F32
           | ((OP == kOpF16 ? 0u : 2u) << 7)          // A format F16 / TF32
           | ((OP == kOpF16 ? 0u : 2u) << 10)         // B format F16 / TF32
           | ((static_cast<uint32_t>(NT) >> 3) << 17)  // N
           | ((256u >> 4) << 24);                     // M
}

// ------------------------------------------------------------- tcgen05 ops --

__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, uint32_t ncols) {
    asm volatile(
        "tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
            smem_addr(dst_smem)),
        "r"(ncols)
        : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::
                     : "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(
                     taddr),
                 "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// One M=256 x N=NT MMA over the CTA pair (K = 8 TF32 or 16 FP16 reals),
// issued by the leader.
template <int OP, int NT>
__device__ __forceinline__ void mma_pair(uint32_t d_tmem, uint64_t a_desc,
                                         uint64_t b_desc, uint32_t accumulate) {
    constexpr uint32_t kIdesc = idesc<OP, NT>();
    if constexpr (OP == kOpF16) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(
                d_tmem),
            "l"(a_desc), "l"(b_desc), "r"(kIdesc), "r"(accumulate)
            : "memory");
    } else {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::2.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(
                d_tmem),
            "l"(a_desc), "l"(b_desc), "r"(kIdesc), "r"(accumulate)
            : "memory");
    }
}

// hi + lo split of v in the operand format.  TF32: lo is left in FP32 (the
// MMA reads its TF32 part).  FP16: both parts rounded to nearest.
__device__ __forceinline__ uint32_t pack_f16x2(float a, float b) {
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
}

// Arrives on `bar` (same offset) in both CTAs of the pair once the MMAs
// issued so far have completed.
__device__ __forceinline__ void mma_commit_pair(uint64_t *bar) {
    const uint16_t mask = 0x3;
    asm volatile(
        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster."
        "multicast::cluster.b64 [%0], %1;" ::"r"(smem_addr(bar)),
        "h"(mask)
        : "memory");
}

__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

__device__ __forceinline__ void cluster_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
                 "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Arrive on the barrier at the same offset in CTA `rank` of the cluster.
__device__ __forceinline__ void mbar_arrive_remote(uint64_t *bar, uint32_t rank) {
    uint32_t remote;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;"
                 : "=r"(remote)
                 : "r"(smem_addr(bar)), "r"(rank));
    asm volatile("mbarrier.arrive.shared::cluster.b64 _, [%0];" ::"r"(remote)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_cluster(uint64_t *bar, uint32_t parity) {
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

// Bounded wait on a barrier that also receives arrivals from the peer CTA.
__device__ __forceinline__ bool mbar_wait_cluster(uint64_t *bar, uint32_t parity,
                                                  unsigned int *err) {
    if (mbar_try_cluster(bar, parity)) return true;
    const uint64_t t0 = global_timer_ns();
    for (uint32_t it = 1;; ++it) {
        if (mbar_try_cluster(bar, parity)) return true;
        if ((it & 15u) == 0u && global_timer_ns() - t0 > kWaitLimitNs) {
            atomicOr(err, kErrWaitTimeout);
            return false;
        }
    }
}

__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

// 32 lanes x 16 consecutive FP32 columns of tensor memory.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]),
          "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
          "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ------------------------------------------------------------------ tables --

struct GridGeom {
    int64_t n[3];        // x, y, z lengths (2-D: y is a dummy axis of length 1)
    int64_t off[3];      // offsets of the axes in the concatenated array
    int src[3];          // caller axis feeding x, y, z (-1: dummy)
    int64_t blocks[3];   // table blocks along x (TX, even count), y (TY), z (NT)
    int tile[3];         // TX, TY, NT with TX * TY = 128
    int64_t n_stages;    // padded modes / modes per stage
    int64_t n_modes;
    int ksteps;          // MMA K-steps per pipeline stage
    int op;              // OperandKind
};

// Per-mode real weight multiplying w = z1 - i z2 (axis x only):
//   kWeightNone       1
//   kWeightArray      weight[j] (summate_fourier's spectrum factor)
//   kWeightProjector  p_c(k_j) = delta_c0 - k_cj k_0j / |k_j|^2 computed from
//                     the unmapped wave vectors `weight` (dim, N), component c
//                     (summate_incompr, generator.py:479-495)
enum WeightMode { kWeightNone = 0, kWeightArray = 1, kWeightProjector = 2 };

struct Weight {
    int mode;
    int comp;
    int dim;
    const double *data;
};

// Element `i` (0..2) of a small parameter array without dynamic indexing
// (which would copy the kernel parameter to local memory).
template <typename T>
__device__ __forceinline__ T pick3(const T (&v)[3], int i) {
    return i == 0 ? v[0] : (i == 1 ? v[1] : v[2]);
}

// Per-mode and per-point inputs of the table kernel.  Mode entry: q = k /
// (2 pi) per axis in FP64 and the weighted amplitudes f z1, f z2.  Point
// entry: the FP64 coordinate.  The tables are O((nx + ny + nz) N) work, so
// their phase q x is formed and reduced to [-1/2, 1/2] turns in FP64 (exact
// reduction, any domain size); only the sincospi of the reduced phase is
// FP32.
struct ModeSplit {
    double q[3];
    float w1, w2;
};

__global__ void grid_prep_kernel(GridGeom g, const double *__restrict__ cov,
                                 const double *__restrict__ z1,
                                 const double *__restrict__ z2,
                                 const double *__restrict__ axes, Weight wgt,
                                 int64_t n_pad_modes, int64_t pt_base1,
                                 int64_t pt_base2, int64_t n_pt_total,
                                 ModeSplit *__restrict__ modes,
                                 double *__restrict__ points,
                                 unsigned int *__restrict__ amp_max) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i < n_pad_modes) {
        ModeSplit m{};
        if (i < g.n_modes) {
            double f = 1.0;
            if (wgt.mode == kWeightArray) {
                f = wgt.data[i];
            } else if (wgt.mode == kWeightProjector) {
                double k2 = 0.0;
                for (int d = 0; d < wgt.dim; ++d) {
                    const double kd = wgt.data[d * g.n_modes + i];
                    k2 += kd * kd;
                }
                f = (wgt.comp == 0 ? 1.0 : 0.0) -
                    wgt.data[wgt.comp * g.n_modes + i] * wgt.data[i] / k2;
            }
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const int src = g.src[a];
                m.q[a] = src >= 0 ? cov[src * g.n_modes + i] * kInv2Pi : 0.0;
            }
            m.w1 = static_cast<float>(f * z1[i]);
            m.w2 = static_cast<float>(f * z2[i]);
            // largest amplitude (non-negative floats order like their bits)
            atomicMax(amp_max, __float_as_uint(fmaxf(fabsf(m.w1), fabsf(m.w2))));
        }
        modes[i] = m;
        return;
    }
    const int64_t p = i - n_pad_modes;
    if (p >= n_pt_total) return;
    const int axis = p < pt_base1 ? 0 : (p < pt_base2 ? 1 : 2);
    const int64_t r = p - (axis == 0 ? 0 : (axis == 1 ? pt_base1 : pt_base2));
    double x = 0.0;
    if (r < pick3(g.n, axis) && pick3(g.src, axis) >= 0)
        x = axes[pick3(g.off, axis) + r];
    points[p] = x;
}

// 2^-e with amp = m 2^e, m in [0.5, 1): scales the amplitudes below 1.
__device__ __forceinline__ int amp_exponent(const unsigned int *amp_max) {
    int e = 0;
    frexpf(__uint_as_float(*amp_max), &e);
    return e;
}

// One thread per (axis point, mode), points fastest.  Axis x
// writes w*Ex * 2^-e (amplitudes normalised below 1), axis y writes Ey
// (complex FP32, blocked [block][stage][mode][tile]); axis z writes the
// pre-split image of [Re Ez, Im Ez] in the operand format: per NT-point
// block and stage, the half of each CTA of a pair (NT / 2 points) is one
// contiguous run of [K-step][hi, lo] blocks in the UMMA canonical K-major
// layout.  The phase q x is formed and reduced to [-1/2, 1/2] turns in FP64
// before the FP32 sincospi.
template <int OP>
__global__ void grid_tables_kernel(GridGeom g, const ModeSplit *__restrict__ modes,
                                   const double *__restrict__ points,
                                   int64_t pt_base1, int64_t pt_base2,
                                   const unsigned int *__restrict__ amp_max,
                                   float2 *__restrict__ wx, float2 *__restrict__ ey,
                                   unsigned char *__restrict__ ez_image) {
    constexpr int kMpk = modes_per_kstep(OP);
    const int axis = blockIdx.z;
    const int mps = kMpk * g.ksteps;   // modes per stage
    const int64_t n_pad_modes = g.n_stages * mps;
    const int tile = pick3(g.tile, axis);
    const int64_t rows = pick3(g.blocks, axis) * tile;
    const int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (idx >= rows * n_pad_modes) return;
    // Points fastest (coalesced writes, one mode per warp), except axis x of
    // 3-D grids: modes fastest within a stage, so each x row's modes of a
    // stage are contiguous ([block][stage][point][mode]) and the generators
    // load two modes of w*Ex per 16-byte load.  A warp reads two x rows
    // there; the 16 Ey rows it reads (and the 32 x rows of a 2-D grid) stay
    // point-fastest, which keeps those loads free of bank conflicts.
    const bool x_modes_fastest = axis == 0 && g.tile[1] > 1;
    int64_t r, j;
    if (!x_modes_fastest) {
        r = idx % rows;
        j = idx / rows;
    } else {
        const int64_t stage = idx / (rows * mps);
        const int64_t rem = idx % (rows * mps);
        r = rem / mps;
        j = stage * mps + rem % mps;
    }

    float c = 0.0f, s = 0.0f;
    const bool live = (j < g.n_modes) && (r < pick3(g.n, axis));
    const ModeSplit &md = modes[j];
    const float w1 = md.w1, w2 = md.w2;
    if (live) {
        const double x = points[(axis == 0 ? 0 : (axis == 1 ? pt_base1 : pt_base2)) + r];
        const double t = pick3(md.q, axis) * x;            // turns
        const float rt = static_cast<float>(t - rint(t));  // exact, in [-1/2, 1/2]
        sincospif(2.0f * rt, &s, &c);
    }
    const int64_t st = j / mps;
    const int mm = static_cast<int>(j % mps);
    const int64_t blk = r / tile;
    const int t = static_cast<int>(r % tile);
    if (axis == 0) {
        // w E with w = f (z1 - i z2), times 2^-e (exact)
        float re = 0.0f, im = 0.0f;
        if (live) {
            const int e = amp_exponent(amp_max);
            re = ldexpf(fmaf(w1, c, w2 * s), -e);
            im = ldexpf(fmaf(w1, s, -w2 * c), -e);
        }
        if (g.tile[1] == 1) {
            // 2-D: the A operand itself, [Re P, -Im P] with P = w Ex, split
            // into hi + lo in the UMMA canonical K-major layout, per
            // 128-row block and stage [K-step][hi, lo] (the generator's
            // layout of a slot)
            const int kstep = mm / kMpk;
            const uint32_t k0 = 2u * (mm % kMpk);
            unsigned char *img = reinterpret_cast<unsigned char *>(wx) +
                                 (blk * g.n_stages + st) *
                                     (static_cast<int64_t>(g.ksteps) * 2 * kBlockBytes);
            unsigned char *ah = img + (kstep * 2 + 0) * kBlockBytes;
            unsigned char *al = img + (kstep * 2 + 1) * kBlockBytes;
            const float vals[2] = {re, -im};
            if constexpr (OP == kOpF16) {
                const __half2 hi = __floats2half2_rn(vals[0], vals[1]);
                const float2 hf = __half22float2(hi);
                const uint32_t o = core_offset(static_cast<uint32_t>(t), k0, OP);
                *reinterpret_cast<__half2 *>(ah + o) = hi;
                *reinterpret_cast<__half2 *>(al + o) =
                    __floats2half2_rn(vals[0] - hf.x, vals[1] - hf.y);
            } else {
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const float hi = to_tf32(vals[q]);
                    const uint32_t o = core_offset(static_cast<uint32_t>(t), k0 + q, OP);
                    *reinterpret_cast<float *>(ah + o) = hi;
                    *reinterpret_cast<float *>(al + o) = vals[q] - hi;
                }
            }
        } else if (x_modes_fastest) {
            wx[((blk * g.n_stages + st) * tile + t) * mps + mm] = make_float2(re, im);
        } else {
            wx[((blk * g.n_stages + st) * mps + mm) * tile + t] = make_float2(re, im);
        }
    } else if (axis == 1) {
        if (g.tile[1] > 1)   // 2-D grids have no y table
            ey[((blk * g.n_stages + st) * mps + mm) * tile + t] = make_float2(c, s);
    } else {
        const int cta_cols = tile / 2;
        const int bblk = b_block_bytes(tile);
        const int rank = t / cta_cols;
        const uint32_t row = static_cast<uint32_t>(t % cta_cols);
        const int kstep = mm / kMpk;
        const uint32_t k0 = 2u * (mm % kMpk);
        const int64_t half_bytes = static_cast<int64_t>(g.ksteps) * 2 * bblk;
        unsigned char *half = ez_image + ((blk * g.n_stages + st) * 2 + rank) * half_bytes;
        unsigned char *bh = half + (kstep * 2 + 0) * bblk;
        unsigned char *bl = half + (kstep * 2 + 1) * bblk;
        if constexpr (OP == kOpF16) {
            // (Re, Im) are adjacent in K: one 4-byte store per part
            const __half2 hi = __floats2half2_rn(c, s);
            const float2 hf = __half22float2(hi);
            const uint32_t o = core_offset(row, k0, OP);
            *reinterpret_cast<__half2 *>(bh + o) = hi;
            *reinterpret_cast<__half2 *>(bl + o) = __floats2half2_rn(c - hf.x, s - hf.y);
        } else {
            const float vals[2] = {c, s};
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const float hi = to_tf32(vals[q]);
                const float lo = to_tf32(vals[q] - hi);
                const uint32_t o = core_offset(row, k0 + q, OP);
                *reinterpret_cast<float *>(bh + o) = hi;
                *reinterpret_cast<float *>(bl + o) = lo;
            }
        }
    }
}

// -------------------------------------------------------------- main kernel --

__device__ __forceinline__ int64_t ceil_div_dev(int64_t a, int64_t b) {
    return (a + b - 1) / b;
}

struct GridArgs {
    GridGeom g;
    int64_t pair_blocks[3];   // pair tiles along x (2 TX), y (TY), z (NT)
    // Work items: the first n_full pair tiles run whole; every later tile is
    // split into `split` (1 or 2) parts over its stages, and the parts add
    // their scaled sums into the (pre-zeroed) output, so the last partial
    // wave of tiles is spread over the idle SM pairs.
    int64_t n_full;
    int split;
    int64_t stages_per_part;
    int64_t tile_offset;   // first pair tile of this launch
    const float2 *wx;
    const float2 *ey;
    const unsigned char *ez_image;
    const unsigned int *amp_max;   // largest |f z|: output scaled by 2^e
    void *out;
    int out_f32;
    double scale;
    unsigned int *err;
};

// One ring of pipeline slots per CTA: its half of B (bulk copy) and its 128
// rows of A: generated from the w*Ex and Ey table slices (bulk copies) on
// 3-D grids, bulk-copied whole on 2-D grids.
template <int TY, int OP, int NT>
struct StageLayout {
    static constexpr int TX = kCtaRows / TY;
    static constexpr bool kACopied = a_copied(TY);
    static constexpr int KS = ksteps_for(TY, OP);
    static constexpr int kModesPerStage = modes_per_stage(TY, OP);
    static constexpr int kChunkStages = chunk_modes(OP) / kModesPerStage;
    static constexpr int kAStageBytes = KS * 2 * kBlockBytes;
    static constexpr int kBStageBytes = KS * 2 * b_block_bytes(NT);   // per CTA
    static constexpr int kWxBytes = kACopied ? 0 : kModesPerStage * TX * 8;
    static constexpr int kEyBytes = kACopied ? 0 : kModesPerStage * TY * 8;
    static constexpr int kB = 0;
    static constexpr int kA = kB + kBStageBytes;
    static constexpr int kWx = kA + kAStageBytes;
    static constexpr int kEy = kWx + kWxBytes;
    static constexpr int kCopyBytes =
        kBStageBytes + (kACopied ? kAStageBytes : kWxBytes + kEyBytes);
    static constexpr int kSlot = (kEy + kEyBytes + 1023) / 1024 * 1024;
    static constexpr int kBudget = 227 * 1024 - 2048;
    static constexpr int kPipe0 = kBudget / kSlot;
    static constexpr int kPipe = kPipe0 > 6 ? 6 : kPipe0;
    static constexpr int kBars = kPipe * kSlot;
    static constexpr int kSmem = kBars + 1024 /*align*/ + 512 /*bars*/;
    static_assert(kPipe >= 3, "ring too shallow");
    static_assert(kPipe * kSlot >= kCtaRows * (NT + 4) * 4,
                  "ring too small to stage a float32 tile");
    static_assert(kChunkStages >= 1, "chunk shorter than a stage");
};

template <int TY, int OP, int NT>
__global__ void __launch_bounds__(kThreads, 1)
    grid_tc_kernel(const GridArgs a) {
    using L = StageLayout<TY, OP, NT>;
    constexpr int kTileCols = NT;
    constexpr int kColsPerThread = NT / 4;   // a quarter of an accumulator row
    constexpr int kBBlock = b_block_bytes(NT);
    constexpr int TX = L::TX;
    constexpr int P = L::kPipe;
    constexpr int KS = L::KS;
    constexpr int kModesPerStage = L::kModesPerStage;
    constexpr int kChunkStages = L::kChunkStages;
    constexpr int kBStageBytes = L::kBStageBytes;

    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L::kBars);
    uint64_t *full = bars;               // [P] local bulk copies landed
    uint64_t *ready = bars + P;          // [P] leader: both halves generated
    uint64_t *empty = bars + 2 * P;      // [P] pair MMAs done with the slot
    uint64_t *gen_done = bars + 3 * P;   // [P] peer: its half generated
    uint64_t *chunk_done = bars + 4 * P; // [2] accumulator complete
    uint64_t *acc_free = chunk_done + 2; // [2] leader: both CTAs drained
    uint64_t *drained = chunk_done + 4;  // [2] peer: its half drained
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(chunk_done + 6);

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t rank = cluster_rank();
    const GridGeom &g = a.g;

    const int64_t item = blockIdx.x >> 1;
    int64_t pair = item, st0 = 0, st1 = g.n_stages;
    bool accumulate_out = false;
    if (item >= a.n_full) {
        const int64_t j = item - a.n_full;
        pair = a.n_full + j / a.split;
        st0 = (j % a.split) * a.stages_per_part;
        st1 = min(st0 + a.stages_per_part, g.n_stages);
        accumulate_out = a.split > 1;
    }
    pair += a.tile_offset;
    const int64_t zb = pair % a.pair_blocks[2];
    const int64_t yb = (pair / a.pair_blocks[2]) % a.pair_blocks[1];
    const int64_t xb = pair / (a.pair_blocks[2] * a.pair_blocks[1]);
    const int64_t xblk = 2 * xb + rank;   // this CTA's TX-row table block
    const int64_t n_all = g.n_stages;         // stages in the tables
    const int64_t n_st = max(st1 - st0, int64_t(0));  // stages of this item
    const int64_t n_chunks = ceil_div_dev(n_st, kChunkStages);

    if (threadIdx.x == 0) {
        // ready / acc_free (leader): 8 local warps + the peer's relay;
        // gen_done / drained (peer): 8 local warps.
        for (int s = 0; s < P; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&ready[s], kGenThreads / 32 + 1);
            mbar_init(&empty[s], 1);
            mbar_init(&gen_done[s], kGenThreads / 32);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&chunk_done[b], 1);
            mbar_init(&acc_free[b], kGenThreads / 32 + 1);
            mbar_init(&drained[b], kGenThreads / 32);
        }
        fence_mbar_init();
    }
    if (warp == 1) tmem_alloc(tmem_slot, kTmemCols);
    tc_fence_before();
    cluster_sync();   // barriers of both CTAs initialised, TMEM allocated
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    bool ok = true;
    // The three single-thread roles run as whole warps: every lane waits,
    // lane 0 issues.  (A warp whose lane 0 loops alone while its other lanes
    // wait to reconverge was measured to slow the generator warps of its
    // SM sub-partition by half.)
    if (warp == 0) {
        // ---------------------------------------------- bulk producer --
        {
            const unsigned char *ez_src =
                a.ez_image + ((zb * n_all + st0) * 2 + rank) * kBStageBytes;
            const float2 *wx_src =
                a.wx + (xblk * n_all + st0) * kModesPerStage * TX;
            const float2 *ey_src = a.ey + (yb * n_all + st0) * kModesPerStage * TY;
            for (int64_t st = 0; st < n_st && ok; ++st) {
                const int s = static_cast<int>(st % P);
                const uint32_t ph = static_cast<uint32_t>((st / P) & 1);
                ok = __shfl_sync(0xffffffffu, mbar_wait(&empty[s], ph ^ 1u, a.err), 0);
                if (!ok) break;
                if (lane == 0) {
                    unsigned char *dst = smem + s * L::kSlot;
                    mbar_arrive_expect_tx(&full[s], L::kCopyBytes);
                    bulk_copy_g2s(dst + L::kB, ez_src + st * 2 * kBStageBytes,
                                  kBStageBytes, &full[s]);
                    if constexpr (L::kACopied) {
                        // the A image of this CTA's 128 rows (2-D grids)
                        const unsigned char *a_src =
                            reinterpret_cast<const unsigned char *>(a.wx) +
                            (xblk * n_all + st0 + st) * L::kAStageBytes;
                        bulk_copy_g2s(dst + L::kA, a_src, L::kAStageBytes, &full[s]);
                    } else {
                        bulk_copy_g2s(dst + L::kWx, wx_src + st * kModesPerStage * TX,
                                      L::kWxBytes, &full[s]);
                        bulk_copy_g2s(dst + L::kEy, ey_src + st * kModesPerStage * TY,
                                      L::kEyBytes, &full[s]);
                    }
                }
                __syncwarp();
            }
        }
    } else if (warp == 1 && rank == 1) {
        // ---------------------------------------- relay (peer only) --
        // Forwards the peer's local "half generated" and "half drained"
        // phases to the leader's ready / acc_free barriers, so the
        // cluster-scope release of a remote arrive is paid by this thread
        // alone, once per phase, instead of by every generator warp.
        // The thread sleeps in try_wait (suspend hint) on the next stage, or
        // once every stage is forwarded on the next chunk, instead of
        // spinning on test_wait beside the generator warps of its SM
        // partition.
        {
            int64_t st = 0, c = 0;
            uint64_t t0 = global_timer_ns();
            while (st < n_st || c < n_chunks) {
                bool moved = false;
                if (st < n_st) {
                    const bool got = __shfl_sync(
                        0xffffffffu,
                        mbar_try_hint(&gen_done[st % P],
                                      static_cast<uint32_t>((st / P) & 1), 200u),
                        0);
                    if (got) {
                        if (lane == 0) mbar_arrive_remote(&ready[st % P], 0);
                        ++st;
                        moved = true;
                    }
                } else {
                    const bool got = __shfl_sync(
                        0xffffffffu,
                        mbar_try_hint(&drained[c & 1],
                                      static_cast<uint32_t>((c >> 1) & 1), 200u),
                        0);
                    if (got) {
                        if (lane == 0) mbar_arrive_remote(&acc_free[c & 1], 0);
                        ++c;
                        moved = true;
                    }
                }
                if (c < n_chunks &&
                    __shfl_sync(0xffffffffu,
                                mbar_test(&drained[c & 1],
                                          static_cast<uint32_t>((c >> 1) & 1)),
                                0)) {
                    if (lane == 0) mbar_arrive_remote(&acc_free[c & 1], 0);
                    ++c;
                    moved = true;
                }
                __syncwarp();
                if (moved) {
                    t0 = global_timer_ns();
                } else if (__shfl_sync(0xffffffffu, global_timer_ns() - t0 > kWaitLimitNs,
                                       0)) {
                    if (lane == 0) atomicOr(a.err, kErrWaitTimeout);
                    break;
                }
            }
        }
    } else if (warp == 1) {
        // ------------------------------------ MMA issuer (leader only) --
        {
            // Descriptor of the ring's first byte; the start-address field
            // (bits 0-13, address / 16) of any operand block is this plus
            // its offset / 16 (shared memory < 256 KB, so it cannot carry).
            const uint64_t desc0 = smem_desc(smem_addr(smem));
            for (int64_t st = 0; st < n_st && ok; ++st) {
                const int s = static_cast<int>(st % P);
                const uint32_t ph = static_cast<uint32_t>((st / P) & 1);
                const int64_t c = st / kChunkStages;
                const int buf = static_cast<int>(c & 1);
                const bool first = (st % kChunkStages) == 0;
                if (first && c >= 2) {
                    // accumulator reused: both CTAs must have drained c - 2
                    ok = __shfl_sync(0xffffffffu,
                                     mbar_wait_cluster(&acc_free[buf],
                                                       static_cast<uint32_t>(
                                                           ((c >> 1) - 1) & 1),
                                                       a.err),
                                     0);
                    if (!ok) break;
                }
                ok = __shfl_sync(0xffffffffu, mbar_wait_cluster(&ready[s], ph, a.err), 0);
                if (!ok) break;
                tc_fence_after();
                if (lane == 0) {
                    const uint64_t slot_desc = desc0 + ((s * L::kSlot) >> 4);
                    const uint32_t d = tmem + buf * 256;
#pragma unroll
                    for (int ks = 0; ks < KS; ++ks) {
                        const uint64_t bh = slot_desc + ((L::kB + (ks * 2 + 0) * kBBlock) >> 4);
                        const uint64_t bl = slot_desc + ((L::kB + (ks * 2 + 1) * kBBlock) >> 4);
                        const uint64_t ah = slot_desc + ((L::kA + (ks * 2 + 0) * kBlockBytes) >> 4);
                        const uint64_t al = slot_desc + ((L::kA + (ks * 2 + 1) * kBlockBytes) >> 4);
                        const uint32_t acc = (first && ks == 0) ? 0u : 1u;
                        mma_pair<OP, NT>(d, ah, bh, acc);
                        mma_pair<OP, NT>(d, ah, bl, 1u);
                        mma_pair<OP, NT>(d, al, bh, 1u);
                    }
                    mma_commit_pair(&empty[s]);
                    if ((st % kChunkStages) == kChunkStages - 1 || st == n_st - 1)
                        mma_commit_pair(&chunk_done[buf]);
                }
                __syncwarp();
            }
        }
    } else {
        // ------------------------------------- A generators + epilogue --
        const int gt = threadIdx.x - 64;       // 0..511
        const int row = gt & (kCtaRows - 1);   // (x, y) row of this CTA's A
        const int part = gt >> 7;              // quarter of the stage's modes
        const int xl = row / TY, yl = row % TY;
        const int q = warp & 3;                // TMEM lane quarter
        const int cq = (warp - 2) >> 2;        // accumulator column quarter
        const uint32_t t_row = tmem + (static_cast<uint32_t>(q * 32) << 16) +
                               cq * kColsPerThread;
        float acc[kColsPerThread];
#pragma unroll
        for (int i = 0; i < kColsPerThread; ++i) acc[i] = 0.0f;
        int64_t n_drained = 0;

        // Adds chunk `c` (accumulator c & 1) into the registers and tells
        // the leader this warp is done with it.
        auto drain = [&](int64_t c) -> bool {
            const int buf = static_cast<int>(c & 1);
            const bool got = __all_sync(
                0xffffffffu,
                mbar_wait(&chunk_done[buf], static_cast<uint32_t>((c >> 1) & 1),
                          a.err));
            if (!got) return false;
            tc_fence_after();
#pragma unroll
            for (int j = 0; j < kColsPerThread / 16; ++j) {
                float v[16];
                tmem_ld16(t_row + buf * 256 + j * 16, v);
#pragma unroll
                for (int i = 0; i < 16; ++i) acc[j * 16 + i] += v[i];
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(rank == 0 ? &acc_free[buf] : &drained[buf]);
            return true;
        };

        for (int64_t st = 0; st < n_st && ok; ++st) {
            const int s = static_cast<int>(st % P);
            const uint32_t ph = static_cast<uint32_t>((st / P) & 1);
            // full[s] of this phase implies the slot was released (empty)
            ok = mbar_wait(&full[s], ph, a.err);
            if (__any_sync(0xffffffffu, !ok)) { ok = false; break; }
            if constexpr (!L::kACopied) {
                unsigned char *slot = smem + s * L::kSlot;
                const float2 *swx = reinterpret_cast<const float2 *>(slot + L::kWx);
                const float2 *sey = reinterpret_cast<const float2 *>(slot + L::kEy);
                // This thread's modes: m0 .. m0 + kMpt - 1 of the stage, i.e.
                // 2 kMpt consecutive reals [Re P, -Im P] of its row of A, stored
                // in runs of kRun reals (at most one 16-byte core-matrix row).
                constexpr int kMpt = kModesPerStage / (kGenThreads / kCtaRows);
                constexpr int kMpk = modes_per_kstep(OP);
                constexpr int kEps = 16 / elem_bytes(OP);    // reals per 16 bytes
                constexpr int kRun = 2 * kMpt < kEps ? 2 * kMpt : kEps;
                const int m0 = part * kMpt;
    #pragma unroll
                for (int sg = 0; sg < 2 * kMpt / kRun; ++sg) {
                    const int mm = m0 + sg * kRun / 2;        // first mode of the run
                    float x[kRun];
    #pragma unroll
                    for (int m = 0; m < kRun / 2; m += 2) {
                        float2 p0, p1;
                        if constexpr (TY > 1) {
                            // two modes of w*Ex per load (mode-fastest rows)
                            const float4 p2 = *reinterpret_cast<const float4 *>(
                                swx + xl * kModesPerStage + mm + m);
                            p0 = make_float2(p2.x, p2.y);
                            p1 = make_float2(p2.z, p2.w);
                        } else {
                            p0 = swx[(mm + m) * TX + xl];
                            p1 = swx[(mm + m + 1) * TX + xl];
                        }
                        const float2 e0 = sey[(mm + m) * TY + yl];
                        const float2 e1 = sey[(mm + m + 1) * TY + yl];
                        x[2 * m] = fmaf(p0.x, e0.x, -p0.y * e0.y);
                        x[2 * m + 1] = -fmaf(p0.x, e0.y, p0.y * e0.x);
                        x[2 * m + 2] = fmaf(p1.x, e1.x, -p1.y * e1.y);
                        x[2 * m + 3] = -fmaf(p1.x, e1.y, p1.y * e1.x);
                    }
                    const int ksg = mm / kMpk;                // its K-step
                    const uint32_t o = core_offset(row, 2u * (mm % kMpk), OP);
                    unsigned char *ah = slot + L::kA + (ksg * 2 + 0) * kBlockBytes + o;
                    unsigned char *al = slot + L::kA + (ksg * 2 + 1) * kBlockBytes + o;
                    if constexpr (OP == kOpF16) {
                        uint32_t h[kRun / 2], l[kRun / 2];
    #pragma unroll
                        for (int i = 0; i < kRun / 2; ++i) {
                            const __half2 hh = __floats2half2_rn(x[2 * i], x[2 * i + 1]);
                            const float2 hf = __half22float2(hh);
                            h[i] = *reinterpret_cast<const uint32_t *>(&hh);
                            l[i] = pack_f16x2(x[2 * i] - hf.x, x[2 * i + 1] - hf.y);
                        }
                        if constexpr (kRun == 8) {
                            *reinterpret_cast<uint4 *>(ah) = make_uint4(h[0], h[1], h[2], h[3]);
                            *reinterpret_cast<uint4 *>(al) = make_uint4(l[0], l[1], l[2], l[3]);
                        } else {
                            *reinterpret_cast<uint2 *>(ah) = make_uint2(h[0], h[1]);
                            *reinterpret_cast<uint2 *>(al) = make_uint2(l[0], l[1]);
                        }
                    } else {
                        static_assert(OP == kOpF16 || kRun == 4, "TF32 runs are 16 bytes");
                        float hi[4], lo[4];
    #pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            hi[i] = to_tf32(x[i]);
                            lo[i] = x[i] - hi[i];   // the MMA reads lo as TF32
                        }
                        *reinterpret_cast<float4 *>(ah) = make_float4(hi[0], hi[1], hi[2], hi[3]);
                        *reinterpret_cast<float4 *>(al) = make_float4(lo[0], lo[1], lo[2], lo[3]);
                    }
                }
                fence_async_smem();
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(rank == 0 ? &ready[s] : &gen_done[s]);
            // Drain a finished chunk as soon as the tensor cores are done
            // with it (one per stage at most).
            if (n_drained < n_chunks) {
                const int buf = static_cast<int>(n_drained & 1);
                const bool done = __shfl_sync(
                    0xffffffffu,
                    lane == 0 ? mbar_test(&chunk_done[buf],
                                          static_cast<uint32_t>((n_drained >> 1) & 1))
                              : false,
                    0);
                if (done) {
                    ok = drain(n_drained);
                    ++n_drained;
                }
            }
        }
        for (; n_drained < n_chunks && ok; ++n_drained) ok = drain(n_drained);

        // Whole float32 tiles leave through shared memory: every thread
        // parks its 64 sums (row q*32+lane, column quarter cq) in the ring,
        // which is idle once the last chunk is drained (all MMAs that read
        // it are complete, all copies consumed), then each warp writes
        // 512 contiguous bytes of one row per store instead of 32 pieces of
        // 16 bytes in 32 rows.  The condition is uniform over the CTA, and
        // every generator thread reaches both barriers (also after a
        // timeout), so the named barrier cannot hang.
        const int64_t nz_all = g.n[2];
        const bool staged = a.out_f32 && !accumulate_out &&
                            (zb + 1) * kTileCols <= nz_all && (nz_all & 3) == 0 &&
                            (reinterpret_cast<uintptr_t>(a.out) & 15u) == 0;
        if (staged) {
            constexpr int kStride = kTileCols + 4;   // floats; conflict-free float4
            float *stage = reinterpret_cast<float *>(smem);
            const float sc = static_cast<float>(ldexp(a.scale, amp_exponent(a.amp_max)));
            if (ok) {
                float *dst = stage + (q * 32 + lane) * kStride + cq * kColsPerThread;
#pragma unroll
                for (int i = 0; i < kColsPerThread; i += 4)
                    *reinterpret_cast<float4 *>(dst + i) =
                        make_float4(sc * acc[i], sc * acc[i + 1], sc * acc[i + 2],
                                    sc * acc[i + 3]);
            }
            asm volatile("bar.sync 1, %0;" ::"n"(kGenThreads) : "memory");
            constexpr int kF4PerRow = kTileCols / 4;              // 64 / 48 / 32
            constexpr int kRowsPerPass = kGenThreads / kF4PerRow;  // 8 / 10 / 16
            const int c4 = gt % kF4PerRow;
            if (gt < kRowsPerPass * kF4PerRow) {
#pragma unroll 4
                for (int r = gt / kF4PerRow; r < kCtaRows; r += kRowsPerPass) {
                    const int64_t x = xblk * TX + r / TY;
                    const int64_t y = yb * TY + r % TY;
                    if (x < g.n[0] && y < g.n[1]) {
                        float *o = static_cast<float *>(a.out) +
                                   (x * g.n[1] + y) * nz_all + zb * kTileCols;
                        reinterpret_cast<float4 *>(o)[c4] = *reinterpret_cast<const float4 *>(
                            stage + r * kStride + 4 * c4);
                    }
                }
            }
        } else if (ok) {
            // this thread's accumulator row is TMEM lane q * 32 + lane
            const int erow = q * 32 + lane;
            const int64_t x = xblk * TX + erow / TY;
            const int64_t y = yb * TY + erow % TY;
            const int64_t nz = g.n[2];
            const int64_t z0 = zb * kTileCols + cq * kColsPerThread;
            if (x < g.n[0] && y < g.n[1] && z0 < nz) {
                const int64_t base = (x * g.n[1] + y) * nz + z0;
                const int64_t nvalid = min(static_cast<int64_t>(kColsPerThread), nz - z0);
                // undo the amplitude normalisation of the tables (2^e, exact)
                const double scale = ldexp(a.scale, amp_exponent(a.amp_max));
                const float sc = static_cast<float>(scale);
                if (accumulate_out) {
                    // part of a split tile: add into the zeroed output
                    if (a.out_f32) {
                        float *o = static_cast<float *>(a.out) + base;
                        if (nvalid == kColsPerThread &&
                            (reinterpret_cast<uintptr_t>(o) & 15u) == 0) {
#pragma unroll
                            for (int i = 0; i < kColsPerThread; i += 4)
                                atomicAdd(reinterpret_cast<float4 *>(o + i),
                                          make_float4(sc * acc[i], sc * acc[i + 1],
                                                      sc * acc[i + 2], sc * acc[i + 3]));
                        } else {
#pragma unroll
                            for (int i = 0; i < kColsPerThread; ++i)
                                if (i < nvalid) atomicAdd(o + i, sc * acc[i]);
                        }
                    } else {
                        double *o = static_cast<double *>(a.out) + base;
#pragma unroll
                        for (int i = 0; i < kColsPerThread; ++i)
                            if (i < nvalid) atomicAdd(o + i, scale * acc[i]);
                    }
                } else if (a.out_f32) {
                    float *o = static_cast<float *>(a.out) + base;
                    if (nvalid == kColsPerThread &&
                        (reinterpret_cast<uintptr_t>(o) & 15u) == 0) {
#pragma unroll
                        for (int i = 0; i < kColsPerThread; i += 4)
                            *reinterpret_cast<float4 *>(o + i) = make_float4(
                                sc * acc[i], sc * acc[i + 1], sc * acc[i + 2],
                                sc * acc[i + 3]);
                    } else {
#pragma unroll
                        for (int i = 0; i < kColsPerThread; ++i)
                            if (i < nvalid) o[i] = sc * acc[i];
                    }
                } else {
                    double *o = static_cast<double *>(a.out) + base;
#pragma unroll
                    for (int i = 0; i < kColsPerThread; ++i)
                        if (i < nvalid) o[i] = scale * acc[i];
                }
            }
        }
    }

    // Neither CTA may leave while its peer can still reach its shared memory
    // (MMA operands, remote arrivals) or tensor memory.
    tc_fence_before();
    cluster_sync();
    if (warp == 1) {
        __syncwarp();
        tc_fence_after();
        tmem_dealloc(tmem, kTmemCols);
    }
}

// Zeroes the output of the split pair tiles (their parts add into it): one
// warp per (tile, row), 32 consecutive z values per store instruction.
__global__ void zero_split_tiles_kernel(GridGeom g, GridArgs a, int64_t first_tile,
                                        int64_t n_tiles, int tx, int ty) {
    const int64_t rows = 2 * static_cast<int64_t>(tx) * ty;
    const int64_t warp_id = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp_id >= n_tiles * rows) return;
    const int64_t r = warp_id % rows;
    const int64_t pair = a.tile_offset + first_tile + warp_id / rows;
    const int64_t zb = pair % a.pair_blocks[2];
    const int64_t yb = (pair / a.pair_blocks[2]) % a.pair_blocks[1];
    const int64_t xb = pair / (a.pair_blocks[2] * a.pair_blocks[1]);
    const int64_t x = xb * 2 * tx + r / ty;
    const int64_t y = yb * ty + r % ty;
    if (x >= g.n[0] || y >= g.n[1]) return;
    const int64_t z0 = zb * g.tile[2];
    const int64_t nz = min(static_cast<int64_t>(g.tile[2]), g.n[2] - z0);
    const int64_t o = (x * g.n[1] + y) * g.n[2] + z0;
    for (int64_t z = lane; z < nz; z += 32) {
        if (a.out_f32)
            static_cast<float *>(a.out)[o + z] = 0.0f;
        else
            static_cast<double *>(a.out)[o + z] = 0.0;
    }
}

template <int TY, int OP, int NT>
cudaError_t launch_grid(const GridArgs &args, int64_t n_pairs, cudaStream_t s) {
    using L = StageLayout<TY, OP, NT>;
    cudaError_t e = cudaFuncSetAttribute(grid_tc_kernel<TY, OP, NT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         L::kSmem);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(static_cast<unsigned>(2 * n_pairs));
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = L::kSmem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, grid_tc_kernel<TY, OP, NT>, args);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

template <int TY, int OP>
cudaError_t launch_grid_nt(const GridArgs &args, int64_t n_pairs, cudaStream_t s) {
    switch (args.g.tile[2]) {
        case 128: return launch_grid<TY, OP, 128>(args, n_pairs, s);
        case 192: return launch_grid<TY, OP, 192>(args, n_pairs, s);
        default: return launch_grid<TY, OP, 256>(args, n_pairs, s);
    }
}

// z tile (MMA N) for an axis of nz points: the fewest tile-times, a tile
// costing max(0.8, NT / 256) of a 256-wide one (below 0.8 the A generation,
// which does not shrink with NT, sets the pace); then the fewest padded
// columns (MMA work); then the wider tile.
int pick_tile_cols(int64_t nz) {
    int best = 256;
    int64_t best_time = ceil_div(nz, 256) * 256, best_pad = ceil_div(nz, 256) * 256;
    for (int nt : {192, 128}) {
        const int64_t time = ceil_div(nz, nt) * std::max(205, nt);
        const int64_t pad = ceil_div(nz, nt) * nt;
        if (time < best_time || (time == best_time && pad < best_pad)) {
            best = nt;
            best_time = time;
            best_pad = pad;
        }
    }
    return best;
}

struct GridPlan {
    GridGeom g;
    int64_t pair_blocks[3];
    int ty;
    int64_t pt_base1, pt_base2, n_pt_total;   // point-split sections
    size_t wx_off, ey_off, ez_off, modes_off, points_off, amp_off, total;
};

int make_plan(int dim, int64_t n_modes, const int64_t *axis_len, GridPlan &p,
              int64_t &total_pts, int op = g_operand_kind.load()) {
    if (dim < 2 || dim > 3) return GST_ERR_UNSUPPORTED_DIM;
    if (axis_len == nullptr || n_modes < 0) return GST_ERR_INVALID_ARGUMENT;
    GridGeom &g = p.g;
    g = GridGeom{};
    int64_t total = 1;
    for (int d = 0; d < dim; ++d) {
        if (axis_len[d] < 0) return GST_ERR_INVALID_ARGUMENT;
        total *= axis_len[d];
    }
    total_pts = total;
    // caller axes -> (x, y, z); a 2-D grid uses a dummy y of length 1
    if (dim == 3) {
        g.src[0] = 0; g.src[1] = 1; g.src[2] = 2;
        g.n[0] = axis_len[0]; g.n[1] = axis_len[1]; g.n[2] = axis_len[2];
        g.off[0] = 0; g.off[1] = axis_len[0]; g.off[2] = axis_len[0] + axis_len[1];
        p.ty = 16;
    } else {
        g.src[0] = 0; g.src[1] = -1; g.src[2] = 1;
        g.n[0] = axis_len[0]; g.n[1] = 1; g.n[2] = axis_len[1];
        g.off[0] = 0; g.off[1] = 0; g.off[2] = axis_len[0];
        p.ty = 1;
    }
    g.tile[0] = kCtaRows / p.ty;
    g.tile[1] = p.ty;
    g.tile[2] = pick_tile_cols(g.n[2]);
    p.pair_blocks[0] = ceil_div(g.n[0], 2 * g.tile[0]);
    p.pair_blocks[1] = ceil_div(g.n[1], g.tile[1]);
    p.pair_blocks[2] = ceil_div(g.n[2], g.tile[2]);
    g.blocks[0] = 2 * p.pair_blocks[0];   // both CTAs of every pair have a block
    g.blocks[1] = p.pair_blocks[1];
    g.blocks[2] = p.pair_blocks[2];
    g.op = op;
    g.ksteps = ksteps_for(p.ty, op);
    const int mps = modes_per_stage(p.ty, op);
    g.n_stages = ceil_div(n_modes, mps);
    g.n_modes = n_modes;
    if (2 * p.pair_blocks[0] * p.pair_blocks[1] * p.pair_blocks[2] > 0x7fffffffLL)
        return GST_ERR_TOO_LARGE;
    const size_t per_stage = mps * sizeof(float2);
    // 2-D: the pre-split A image (per 128-row block and stage) instead of
    // the w*Ex table, and no y table
    const size_t wx_bytes =
        a_copied(p.ty) ? static_cast<size_t>(g.blocks[0]) * g.n_stages * g.ksteps * 2 *
                             kBlockBytes
                       : static_cast<size_t>(g.blocks[0]) * g.n_stages * per_stage *
                             g.tile[0];
    const size_t ey_bytes = a_copied(p.ty) ? 0
                                           : static_cast<size_t>(g.blocks[1]) *
                                                 g.n_stages * per_stage * g.tile[1];
    const size_t ez_bytes = static_cast<size_t>(g.blocks[2]) * g.n_stages * 2 *
                            g.ksteps * 2 * b_block_bytes(g.tile[2]);
    p.pt_base1 = g.blocks[0] * g.tile[0];
    p.pt_base2 = p.pt_base1 + g.blocks[1] * g.tile[1];
    p.n_pt_total = p.pt_base2 + g.blocks[2] * g.tile[2];
    p.ez_off = 0;
    p.wx_off = align_up(ez_bytes, 256);
    p.ey_off = align_up(p.wx_off + wx_bytes, 256);
    p.modes_off = align_up(p.ey_off + ey_bytes, 256);
    p.points_off = align_up(p.modes_off + sizeof(ModeSplit) * g.n_stages * mps, 256);
    p.amp_off = align_up(p.points_off + sizeof(double) * p.n_pt_total, 256);
    p.total = p.amp_off + sizeof(unsigned int);
    return GST_OK;
}

int run_tables(const GridPlan &p, const double *axes, const double *cov,
               const double *z1, const double *z2, unsigned char *ws,
               cudaStream_t s, Weight wgt = Weight{kWeightNone, 0, 0, nullptr}) {
    const GridGeom &g = p.g;
    const int64_t n_pad_modes = g.n_stages * modes_per_stage(p.ty, g.op);
    ModeSplit *modes = reinterpret_cast<ModeSplit *>(ws + p.modes_off);
    double *points = reinterpret_cast<double *>(ws + p.points_off);
    unsigned int *amp = reinterpret_cast<unsigned int *>(ws + p.amp_off);
    const int threads = 256;
    GST_TRY_CUDA(cudaMemsetAsync(amp, 0, sizeof(unsigned int), s));
    grid_prep_kernel<<<static_cast<unsigned>(ceil_div(n_pad_modes + p.n_pt_total, threads)),
                       threads, 0, s>>>(g, cov, z1, z2, axes, wgt, n_pad_modes,
                                        p.pt_base1, p.pt_base2, p.n_pt_total, modes,
                                        points, amp);
    GST_TRY_CUDA(cudaGetLastError());
    int64_t max_rows = 0;
    for (int d = 0; d < 3; ++d)
        max_rows = std::max(max_rows, g.blocks[d] * g.tile[d]);
    const dim3 grid(static_cast<unsigned>(ceil_div(max_rows * n_pad_modes, threads)),
                    1, 3);
    auto *tables = g.op == kOpF16 ? grid_tables_kernel<kOpF16>
                                  : grid_tables_kernel<kOpTf32>;
    tables<<<grid, threads, 0, s>>>(g, modes, points, p.pt_base1, p.pt_base2, amp,
                                    reinterpret_cast<float2 *>(ws + p.wx_off),
                                    reinterpret_cast<float2 *>(ws + p.ey_off),
                                    ws + p.ez_off);
    GST_TRY_CUDA(cudaGetLastError());
    return GST_OK;
}

int run_contract(const GridPlan &p, const unsigned char *ws, void *out,
                 int out_type, double scale, cudaStream_t s,
                 int64_t tile_begin = 0, int64_t tile_end = -1) {
    unsigned int *err = device_error_word();
    if (err == nullptr) return GST_ERR_CUDA;
    GridArgs args{};
    args.g = p.g;
    for (int d = 0; d < 3; ++d) args.pair_blocks[d] = p.pair_blocks[d];
    args.wx = reinterpret_cast<const float2 *>(ws + p.wx_off);
    args.ey = reinterpret_cast<const float2 *>(ws + p.ey_off);
    args.ez_image = ws + p.ez_off;
    args.amp_max = reinterpret_cast<const unsigned int *>(ws + p.amp_off);
    args.out = out;
    args.out_f32 = out_type == GST_OUT_F32 ? 1 : 0;
    args.scale = scale;
    args.err = err;
    const int64_t all_tiles = p.pair_blocks[0] * p.pair_blocks[1] * p.pair_blocks[2];
    if (tile_end < 0 || tile_end > all_tiles) tile_end = all_tiles;
    if (tile_begin >= tile_end) return GST_OK;
    const int64_t n_tiles = tile_end - tile_begin;
    args.tile_offset = tile_begin;
    // Tiles of the last partial wave are split in two over their stages
    // when that fits in the idle SM pairs (two parts per tile keep the sum
    // order-independent: both add into an exact zero).
    const int64_t slots = std::max(1, sm_count() / 2);
    const int64_t tail = n_tiles % slots;
    int split = 1;
    if (tail > 0 && 2 * tail <= slots && p.g.n_stages >= 2) split = 2;
    // Outputs in host memory (zero-copy over the C2C link) get plain stores
    // only: no split tiles, hence no atomics on host memory.
    cudaPointerAttributes attr{};
    if (cudaPointerGetAttributes(&attr, out) == cudaSuccess &&
        attr.type == cudaMemoryTypeHost)
        split = 1;
    cudaGetLastError();  // an unregistered pointer leaves an error behind
    args.split = split;
    args.n_full = split > 1 ? n_tiles - tail : n_tiles;
    args.stages_per_part = ceil_div(p.g.n_stages, split);
    if (split > 1) {
        const int tx = p.g.tile[0], ty = p.g.tile[1];
        const int64_t warps = tail * 2 * tx * ty;   // one per (tile, row)
        const int blocks = static_cast<int>(ceil_div(warps * 32, 256));
        zero_split_tiles_kernel<<<blocks, 256, 0, s>>>(p.g, args, args.n_full, tail,
                                                       tx, ty);
        GST_TRY_CUDA(cudaGetLastError());
    }
    const int64_t n_items = args.n_full + (n_tiles - args.n_full) * split;
    cudaError_t e;
    if (p.g.op == kOpF16)
        e = (p.ty == 16) ? launch_grid_nt<16, kOpF16>(args, n_items, s)
                         : launch_grid_nt<1, kOpF16>(args, n_items, s);
    else
        e = (p.ty == 16) ? launch_grid_nt<16, kOpTf32>(args, n_items, s)
                         : launch_grid_nt<1, kOpTf32>(args, n_items, s);
    GST_TRY_CUDA(e);
    return GST_OK;
}

bool valid_out(int t) { return t == GST_OUT_F64 || t == GST_OUT_F32; }

}  // namespace
}  // namespace gst

extern "C" {

int gst_grid_tc_set_operands(int kind) {
    if (kind != GST_TC_TF32 && kind != GST_TC_F16) return -1;
    return gst::g_operand_kind.exchange(kind);
}

int gst_grid_tc_tile_cols(int64_t nz) {
    return nz < 0 ? -1 : gst::pick_tile_cols(nz);
}

int gst_grid_tc_workspace_size(int dim, int64_t n_modes,
                               const int64_t *axis_len, size_t *bytes) {
    if (bytes == nullptr) return GST_ERR_INVALID_ARGUMENT;
    gst::GridPlan p;
    int64_t total = 0;
    const int rc = gst::make_plan(dim, n_modes, axis_len, p, total);
    if (rc) return rc;
    *bytes = (total == 0 || n_modes == 0) ? 0 : p.total;
    return GST_OK;
}

int gst_grid_tc_tables(int dim, int64_t n_modes, const int64_t *axis_len,
                       const double *axes, const double *cov_samples,
                       const double *z_1, const double *z_2, void *workspace,
                       size_t workspace_bytes, void *stream) {
    gst::GridPlan p;
    int64_t total = 0;
    int rc = gst::make_plan(dim, n_modes, axis_len, p, total);
    if (rc) return rc;
    if (total == 0 || n_modes == 0) return GST_OK;
    if (workspace == nullptr || workspace_bytes < p.total || axes == nullptr ||
        cov_samples == nullptr || z_1 == nullptr || z_2 == nullptr)
        return GST_ERR_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(workspace) % 256 != 0)
        return GST_ERR_ALIGNMENT;
    if (gst::current_device() < 0) return GST_ERR_NO_DEVICE;
    return gst::run_tables(p, axes, cov_samples, z_1, z_2,
                           static_cast<unsigned char *>(workspace),
                           static_cast<cudaStream_t>(stream));
}

int gst_grid_tc_contract(int dim, int64_t n_modes, const int64_t *axis_len,
                         const void *workspace, size_t workspace_bytes,
                         void *out, int out_type, double scale, void *stream) {
    if (!gst::valid_out(out_type)) return GST_ERR_INVALID_ARGUMENT;
    gst::GridPlan p;
    int64_t total = 0;
    int rc = gst::make_plan(dim, n_modes, axis_len, p, total);
    if (rc) return rc;
    if (total == 0) return GST_OK;
    if (out == nullptr) return GST_ERR_INVALID_ARGUMENT;
    if (gst::current_device() < 0) return GST_ERR_NO_DEVICE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n_modes == 0) {
        const size_t elem = out_type == GST_OUT_F32 ? 4 : 8;
        GST_TRY_CUDA(cudaMemsetAsync(out, 0, elem * total, s));
        return GST_OK;
    }
    if (workspace == nullptr || workspace_bytes < p.total)
        return GST_ERR_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(workspace) % 256 != 0)
        return GST_ERR_ALIGNMENT;
    return gst::run_contract(p, static_cast<const unsigned char *>(workspace),
                             out, out_type, scale, s);
}

// Shared driver of the weighted grid entry points: n_comp weighted
// contractions into consecutive output blocks, one workspace.
static int weighted_grid(int dim, int64_t n_modes, const int64_t *axis_len,
                         const double *axes, const double *cov, const double *z1,
                         const double *z2, gst::Weight wgt, int n_comp, void *out,
                         int out_type, double scale, void *stream) {
    if (!gst::valid_out(out_type)) return GST_ERR_INVALID_ARGUMENT;
    gst::GridPlan p;
    int64_t total = 0;
    int rc = gst::make_plan(dim, n_modes, axis_len, p, total);
    if (rc) return rc;
    if (total == 0) return GST_OK;
    if (out == nullptr) return GST_ERR_INVALID_ARGUMENT;
    if (gst::current_device() < 0) return GST_ERR_NO_DEVICE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t elem = out_type == GST_OUT_F32 ? 4 : 8;
    if (n_modes == 0) {
        GST_TRY_CUDA(cudaMemsetAsync(out, 0, elem * total * n_comp, s));
        return GST_OK;
    }
    if (cov == nullptr || z1 == nullptr || z2 == nullptr || axes == nullptr ||
        wgt.data == nullptr)
        return GST_ERR_INVALID_ARGUMENT;
    gst::StreamScratch ws;
    GST_TRY_CUDA(ws.alloc(p.total, s));
    unsigned char *base = static_cast<unsigned char *>(ws.ptr);
    for (int c = 0; c < n_comp; ++c) {
        wgt.comp = c;
        rc = gst::run_tables(p, axes, cov, z1, z2, base, s, wgt);
        if (rc) return rc;
        rc = gst::run_contract(p, base,
                               static_cast<unsigned char *>(out) + elem * total * c,
                               out_type, scale, s);
        if (rc) return rc;
    }
    return GST_OK;
}

// Host-memory variant of weighted_grid: copies the inputs in, computes every
// component in x slabs and copies each finished slab to `out` on the
// library's copy stream while the next slab computes.  `out` in pinned
// memory gives asynchronous copies; the call is ordered on `stream` (the
// output is complete once `stream` is).
static int weighted_grid_host(int dim, int64_t n_modes, const int64_t *axis_len,
                              const double *axes, const double *cov,
                              const double *z1, const double *z2,
                              gst::Weight wgt, int64_t wgt_len, int n_comp,
                              void *out, int out_type, double scale,
                              void *stream) {
    if (!gst::valid_out(out_type)) return GST_ERR_INVALID_ARGUMENT;
    gst::GridPlan p;
    int64_t total = 0;
    int rc = gst::make_plan(dim, n_modes, axis_len, p, total);
    if (rc) return rc;
    if (total == 0) return GST_OK;
    if (out == nullptr) return GST_ERR_INVALID_ARGUMENT;
    if (gst::current_device() < 0) return GST_ERR_NO_DEVICE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t elem = out_type == GST_OUT_F32 ? 4 : 8;
    const size_t comp_bytes = elem * static_cast<size_t>(total);
    if (n_modes == 0) {
        GST_TRY_CUDA(cudaStreamSynchronize(s));
        memset(out, 0, comp_bytes * n_comp);
        return GST_OK;
    }
    if (cov == nullptr || z1 == nullptr || z2 == nullptr || axes == nullptr ||
        (wgt.mode != gst::kWeightNone && wgt.data == nullptr))
        return GST_ERR_INVALID_ARGUMENT;
    cudaStream_t cs = gst::copy_stream();
    if (cs == nullptr) return GST_ERR_CUDA;
    // One scratch block: inputs | tables workspace | device field.
    int64_t n_axis = 0;
    for (int d = 0; d < dim; ++d) n_axis += axis_len[d];
    const int64_t n_in = n_axis + (dim + 2) * n_modes +
                         (wgt.mode != gst::kWeightNone ? wgt_len : 0);
    const size_t in_bytes = gst::align_up(8 * static_cast<size_t>(n_in), 256);
    const size_t ws_bytes = gst::align_up(p.total, 256);
    gst::StreamScratch scratch;
    GST_TRY_CUDA(scratch.alloc(in_bytes + ws_bytes + comp_bytes * n_comp, s));
    unsigned char *base = static_cast<unsigned char *>(scratch.ptr);
    double *d_in = reinterpret_cast<double *>(base);
    unsigned char *ws = base + in_bytes;
    unsigned char *field = ws + ws_bytes;
    double *d_axes = d_in, *d_cov = d_axes + n_axis, *d_z1 = d_cov + dim * n_modes;
    double *d_z2 = d_z1 + n_modes, *d_w = d_z2 + n_modes;
    GST_TRY_CUDA(cudaMemcpyAsync(d_axes, axes, 8 * n_axis, cudaMemcpyHostToDevice, s));
    GST_TRY_CUDA(cudaMemcpyAsync(d_cov, cov, 8 * dim * n_modes,
                                 cudaMemcpyHostToDevice, s));
    GST_TRY_CUDA(cudaMemcpyAsync(d_z1, z1, 8 * n_modes, cudaMemcpyHostToDevice, s));
    GST_TRY_CUDA(cudaMemcpyAsync(d_z2, z2, 8 * n_modes, cudaMemcpyHostToDevice, s));
    if (wgt.mode != gst::kWeightNone) {
        GST_TRY_CUDA(cudaMemcpyAsync(d_w, wgt.data, 8 * wgt_len,
                                     cudaMemcpyHostToDevice, s));
        wgt.data = d_w;
    }
    // Slabs: whole pair blocks along x; about 16 MiB each, at most 4 per
    // component (measured on GB300 for a 64 MiB field: 4 slabs end 0.2 ms
    // sooner than one contraction followed by one copy).
    const int64_t xb = 2 * static_cast<int64_t>(p.g.tile[0]);
    const int64_t x_blocks = gst::ceil_div(p.g.n[0], xb);
    const int64_t per_x = p.pair_blocks[1] * p.pair_blocks[2];
    const int64_t row_bytes = static_cast<int64_t>(comp_bytes) / p.g.n[0];
    const int64_t want = std::max<int64_t>(1, static_cast<int64_t>(comp_bytes >> 24));
    const int64_t n_slabs = std::min<int64_t>(std::min<int64_t>(want, 4), x_blocks);
    constexpr int kMaxEvents = 3 * 4;
    cudaEvent_t ev[kMaxEvents + 1] = {};
    int n_ev = 0;
    rc = GST_OK;
    for (int c = 0; c < n_comp && rc == GST_OK; ++c) {
        wgt.comp = c;
        rc = gst::run_tables(p, d_axes, d_cov, d_z1, d_z2, ws, s, wgt);
        for (int64_t k = 0; k < n_slabs && rc == GST_OK; ++k) {
            const int64_t b0 = x_blocks * k / n_slabs, b1 = x_blocks * (k + 1) / n_slabs;
            unsigned char *dst = field + comp_bytes * c;
            rc = gst::run_contract(p, ws, dst, out_type, scale, s, b0 * per_x,
                                   b1 * per_x);
            if (rc) break;
            const int64_t x0 = b0 * xb, x1 = std::min(b1 * xb, p.g.n[0]);
            cudaError_t e = cudaEventCreateWithFlags(&ev[n_ev], cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaEventRecord(ev[n_ev], s);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, ev[n_ev], 0);
            ++n_ev;
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(static_cast<unsigned char *>(out) + comp_bytes * c +
                                        row_bytes * x0,
                                    dst + row_bytes * x0, row_bytes * (x1 - x0),
                                    cudaMemcpyDeviceToHost, cs);
            if (e != cudaSuccess) {
                gst::note_cuda_error(e);
                rc = GST_ERR_CUDA;
            }
        }
    }
    // `stream` waits for the copies before the scratch goes back to the pool.
    cudaError_t e = cudaEventCreateWithFlags(&ev[n_ev], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(ev[n_ev], cs);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ev[n_ev], 0);
    ++n_ev;
    for (int i = 0; i < n_ev; ++i)
        if (ev[i]) cudaEventDestroy(ev[i]);
    if (e != cudaSuccess && rc == GST_OK) {
        gst::note_cuda_error(e);
        rc = GST_ERR_CUDA;
    }
    return rc;
}

int gst_summate_grid_tc_host(int dim, int64_t n_modes, const int64_t *axis_len,
                             const double *axes, const double *cov_samples,
                             const double *z_1, const double *z_2, void *out,
                             int out_type, double scale, void *stream) {
    gst::Weight w{gst::kWeightNone, 0, dim, nullptr};
    return weighted_grid_host(dim, n_modes, axis_len, axes, cov_samples, z_1, z_2,
                              w, 0, 1, out, out_type, scale, stream);
}

int gst_summate_incompr_grid_tc_host(int dim, int64_t n_modes,
                                     const int64_t *axis_len, const double *axes,
                                     const double *cov_samples,
                                     const double *proj_cov, const double *z_1,
                                     const double *z_2, void *out, int out_type,
                                     double scale, void *stream) {
    if (dim < 2 || dim > 3) return GST_ERR_UNSUPPORTED_DIM;
    gst::Weight w{gst::kWeightProjector, 0, dim,
                  proj_cov ? proj_cov : cov_samples};
    return weighted_grid_host(dim, n_modes, axis_len, axes, cov_samples, z_1, z_2,
                              w, dim * n_modes, dim, out, out_type, scale, stream);
}

int gst_summate_fourier_grid_tc_host(int dim, int64_t n_modes,
                                     const int64_t *axis_len, const double *axes,
                                     const double *spectrum_factor,
                                     const double *modes, const double *z_1,
                                     const double *z_2, void *out, int out_type,
                                     double scale, void *stream) {
    gst::Weight w{gst::kWeightArray, 0, dim, spectrum_factor};
    return weighted_grid_host(dim, n_modes, axis_len, axes, modes, z_1, z_2, w,
                              n_modes, 1, out, out_type, scale, stream);
}

int gst_summate_incompr_grid_tc(int dim, int64_t n_modes, const int64_t *axis_len,
                                const double *axes, const double *cov_samples,
                                const double *proj_cov, const double *z_1,
                                const double *z_2, void *out, int out_type,
                                double scale, void *stream) {
    if (dim < 2 || dim > 3) return GST_ERR_UNSUPPORTED_DIM;
    gst::Weight w{gst::kWeightProjector, 0, dim,
                  proj_cov ? proj_cov : cov_samples};
    return weighted_grid(dim, n_modes, axis_len, axes, cov_samples, z_1, z_2, w,
                         dim, out, out_type, scale, stream);
}

int gst_summate_fourier_grid_tc(int dim, int64_t n_modes, const int64_t *axis_len,
                                const double *axes, const double *spectrum_factor,
                                const double *modes, const double *z_1,
                                const double *z_2, void *out, int out_type,
                                double scale, void *stream) {
    gst::Weight w{gst::kWeightArray, 0, dim, spectrum_factor};
    return weighted_grid(dim, n_modes, axis_len, axes, modes, z_1, z_2, w, 1, out,
                         out_type, scale, stream);
}

int gst_grid_tc_contract_rows(int dim, int64_t n_modes, const int64_t *axis_len,
                              const void *workspace, size_t workspace_bytes,
                              void *out, int out_type, double scale,
                              int64_t x_begin, int64_t x_end, void *stream) {
    if (!gst::valid_out(out_type)) return GST_ERR_INVALID_ARGUMENT;
    gst::GridPlan p;
    int64_t total = 0;
    int rc = gst::make_plan(dim, n_modes, axis_len, p, total);
    if (rc) return rc;
    const int64_t xb = 2 * static_cast<int64_t>(p.g.tile[0]);   // pair x rows
    if (x_begin < 0 || x_end < x_begin || x_end > p.g.n[0] || x_begin % xb != 0 ||
        (x_end % xb != 0 && x_end != p.g.n[0]))
        return GST_ERR_INVALID_ARGUMENT;
    if (total == 0 || x_begin == x_end) return GST_OK;
    if (out == nullptr) return GST_ERR_INVALID_ARGUMENT;
    if (gst::current_device() < 0) return GST_ERR_NO_DEVICE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t elem = out_type == GST_OUT_F32 ? 4 : 8;
    const int64_t row_elems = total / p.g.n[0];
    if (n_modes == 0) {
        GST_TRY_CUDA(cudaMemsetAsync(static_cast<unsigned char *>(out) +
                                         elem * row_elems * x_begin,
                                     0, elem * row_elems * (x_end - x_begin), s));
        return GST_OK;
    }
    if (workspace == nullptr || workspace_bytes < p.total)
        return GST_ERR_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(workspace) % 256 != 0)
        return GST_ERR_ALIGNMENT;
    const int64_t per_x = p.pair_blocks[1] * p.pair_blocks[2];
    return gst::run_contract(p, static_cast<const unsigned char *>(workspace), out,
                             out_type, scale, s, (x_begin / xb) * per_x,
                             gst::ceil_div(x_end, xb) * per_x);
}

int gst_summate_grid_tc(int dim, int64_t n_modes, const int64_t *axis_len,
                        const double *axes, const double *cov_samples,
                        const double *z_1, const double *z_2, void *out,
                        int out_type, double scale, void *stream) {
    if (!gst::valid_out(out_type)) return GST_ERR_INVALID_ARGUMENT;
    gst::GridPlan p;
    int64_t total = 0;
    int rc = gst::make_plan(dim, n_modes, axis_len, p, total);
    if (rc) return rc;
    if (total == 0) return GST_OK;
    if (out == nullptr) return GST_ERR_INVALID_ARGUMENT;
    if (gst::current_device() < 0) return GST_ERR_NO_DEVICE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n_modes == 0) {
        const size_t elem = out_type == GST_OUT_F32 ? 4 : 8;
        GST_TRY_CUDA(cudaMemsetAsync(out, 0, elem * total, s));
        return GST_OK;
    }
    if (cov_samples == nullptr || z_1 == nullptr || z_2 == nullptr ||
        axes == nullptr)
        return GST_ERR_INVALID_ARGUMENT;
    gst::StreamScratch ws;
    GST_TRY_CUDA(ws.alloc(p.total, s));
    unsigned char *base = static_cast<unsigned char *>(ws.ptr);
    rc = gst::run_tables(p, axes, cov_samples, z_1, z_2, base, s);
    if (rc) return rc;
    return gst::run_contract(p, base, out, out_type, scale, s);
}

}  // extern "C"
