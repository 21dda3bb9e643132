// k_tc.cu -- coarse cross term on the 5th-generation tensor cores (tcgen05),
// the "precision form" of the coarse pass: BF16 operands, FP32 accumulation
// in tensor memory (TMEM).
//
//   C[r][(p,t)] = sum_k A[r][k] Y[(p,t)][k],  A = projections (BF16 table),
//   Y = m C X E formed on the fly from FP32 b = m C X and the phase table E,
// then diff2 - c_p = N(r,p) - 2 C, stored like the FP32 path (k_gemm.cu) with
// the per-particle minimum.  The coarse pass only decides which poses are
// significant; every significant pose is re-evaluated in FP32 by the fine pass.
//
// Operand tiles are pre-packed in HBM in the exact shared-memory image of a
// canonical no-swizzle K-major layout (8 x 16-byte core matrices; K-adjacent
// core matrices 128 B apart, 8-row groups 1024 B apart): the projection
// table once per iteration (k_pack_a), Y once per batch (k_pack_y).
// Persistent kernel, one 384-thread CTA per SM looping over output tiles of
// 128 (orientations) x 256 (particle, translation); K tiles of 64 BF16 in a
// 4-stage shared-memory ring.  One thread streams each stage's 48 KB with two
// cp.async.bulk copies, one thread issues tcgen05.mma (M=128, N=256, K=16)
// into one of two TMEM accumulators (2 x 256 columns) while eight warps drain
// the other, so the epilogue of tile i overlaps the MMAs of tile i+1.  Every
// mbarrier wait is bounded: on timeout the CTA records an error, waits
// (bounded) for its own copies and MMAs, frees its tensor memory and returns.
#include "gbr_internal.h"

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <cfloat>
#include <algorithm>
#include <cstdint>

namespace gbr {
namespace {

constexpr int TM = 128, TN = 256, TK = 64, STAGES = 4;
constexpr int EPI_WARPS = 8, THREADS = 128 + 32 * EPI_WARPS;
constexpr int A_BYTES = TM * TK * 2;          // 16 KB
constexpr int B_BYTES = TN * TK * 2;          // 32 KB
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int TRANSPOSE_BYTES = EPI_WARPS * 32 * 33 * 4;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + TRANSPOSE_BYTES;
constexpr int TMEM_COLS = 2 * TN;             // two accumulators
constexpr int kGroupMDefault = 32;
constexpr unsigned int kWaitLimit = 1u << 22;

__device__ int g_tc_error;  // first failure code of the last launches (0 = ok)

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (tcgen05): start >> 4, LBO >> 4, SBO >> 4,
// descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major.
__host__ __device__ constexpr uint32_t make_idesc() {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);
}

// Instruction descriptor, kind::tf32: D = F32, A = B = TF32, both K-major.
__host__ __device__ constexpr uint32_t make_idesc_tf32() {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TN >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (unsigned int it = 0; it < kWaitLimit; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ unsigned int f2ord(float f) {
    unsigned int u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t *>(&h);
}

// Byte offset of the 16-byte chunk (row, kg) in a no-swizzle K-major tile
// with TK/8 = 8 core matrices along K.
__device__ __forceinline__ uint32_t chunk_off(int row, int kg) {
    return (uint32_t)((((row >> 3) * (TK / 8) + kg) << 7) + ((row & 7) << 4));
}

__device__ __forceinline__ bool arrive_expect_tx(uint32_t bar, uint32_t bytes) {
    uint64_t state;
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 %0, [%1], %2;"
                 : "=l"(state)
                 : "r"(bar), "r"(bytes)
                 : "memory");
    return state != 0ull || true;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

// The same copy with an L2 cache policy (createpolicy) attached to its reads.
__device__ __forceinline__ void bulk_g2s_hint(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar,
                                              uint64_t policy) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
            dst),
        "l"(src), "r"(bytes), "r"(bar), "l"(policy)
        : "memory");
}

// L2 policy that keeps the lines it reads ahead of normal lines on eviction.
__device__ __forceinline__ uint64_t policy_keep() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

struct TcArgs {
    const uint8_t *Ablk;     // [mtiles][ktiles][A_BYTES] BF16 tiles in shared-memory image
    const uint8_t *Yblk;     // [ntiles][ktiles][B_BYTES]
    int M, ktiles, T, N, nparticles;
    int mtiles, ntiles;
    float *out;              // [p][M][T]
    const float *norm;       // [p][M]
    const float *pdf_orient; // [M]
    ParticleState *ps;
    unsigned int *rowmin;    // [p][M] ordered minimum of each orientation row, or null
    // sparse diff2 writes (null = write every pose): only row segments (the
    // part of an orientation row inside one 32-column chunk) whose minimum is
    // within ps[p].xs of the particle's running minimum are stored, and bit
    // (chunk - first chunk of the row) of segmask[p][M] records them
    unsigned int *segmask;
    int group_m;             // orientation tiles per group of the tile order (>= 1)
    int keep_a;              // read the A tiles with an L2 keep policy
};

// Tile order of the persistent loop: groups of group_m orientation tiles,
// orientation tile fastest inside a group, so that the CTAs running at the
// same time share the group's A tiles (held in L2) and sweep the Y tiles
// once per group: DRAM reads A once and Y ceil(mtiles / group_m) times.
__device__ __forceinline__ void tile_mn(int tidx, int group_m, int mtiles, int ntiles, int &mt, int &nt) {
    const int per_group = group_m * ntiles;
    const int g = tidx / per_group, r = tidx - g * per_group;
    const int gm = min(group_m, mtiles - g * group_m);
    mt = g * group_m + r % gm;
    nt = r / gm;
}

// Warp minimum of lmin into *dst; returns it (ordered encoding, ~0 = none).
__device__ __forceinline__ unsigned int warp_min_flush(float lmin, unsigned int *dst) {
    const unsigned int u = lmin < __int_as_float(0x7f800000) ? f2ord(lmin) : 0xFFFFFFFFu;
    const unsigned int wmin = __reduce_min_sync(0xffffffffu, u);
    if ((threadIdx.x & 31) == 0 && wmin != 0xFFFFFFFFu) atomicMin(dst, wmin);
    return wmin;
}

__device__ __forceinline__ float ord2f(unsigned int u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Near cut of a particle from its running minimum diff2 (ordered encoding,
// never below the final minimum) and its skip distance xs; -inf while it has
// no finite diff2 yet.  A segment whose minimum is above the cut is above
// final minimum + xs too.
__device__ __forceinline__ float near_cut(unsigned int run, float xs) {
    if (run == 0xFFFFFFFFu) return -__int_as_float(0x7f800000);
    return ord2f(run) + xs + 1.f;  // +1: margin over the readers' float test
}

// Ordered minimum of lane row m for particle p into rowmin (one atomic per
// lane and particle segment of the tile half).
__device__ __forceinline__ void rowmin_flush(const TcArgs &a, int p, int m, float v) {
    if (p >= 0 && v < FLT_MAX) atomicMin(&a.rowmin[(size_t)p * a.M + m], f2ord(v));
}

// Particles a warp's 128 columns can touch when T >= 32.
constexpr int kTileParticles = 128 / 32 + 1;

// Five per-particle values of a tile held in registers (selects, not an
// indexed array, which would live in local memory); get(i) of i outside
// 0..4 returns the last.
template <typename V>
struct TileOps {
    V v0, v1, v2, v3, v4;
    __device__ __forceinline__ void set(int i, V x) {
        if (i == 0) v0 = x;
        else if (i == 1) v1 = x;
        else if (i == 2) v2 = x;
        else if (i == 3) v3 = x;
        else v4 = x;
    }
    __device__ __forceinline__ V get(int i) const {
        return i == 0 ? v0 : i == 1 ? v1 : i == 2 ? v2 : i == 3 ? v3 : v4;
    }
};
static_assert(kTileParticles == 5, "TileOps holds five values");

// Epilogue of one cross-term tile: drains the 128 x 256 FP32 accumulator at
// TMEM address acc (rows m0.., columns n0..) into diff2 = N(r,p) - 2 C with
// the particles' running minima, row minima and sparse segment stores.  Warp
// q = warp & 3 reads TMEM lanes 32 q.. (rows m0 + 32 q + lane), h the column
// half 128 h..; tb is the warp's 32 x 33 transpose buffer.
__device__ __forceinline__ void drain_cross(const TcArgs &a, uint32_t acc, int m0, int n0, int q, int h, int lane,
                                            float *tb) {
    const int m = m0 + q * 32 + lane;
    const bool skip = !(m < a.M) || !(a.pdf_orient[m] > 0.f);
    // running row minimum of the particle segment this lane is in
    const bool track_rows = a.rowmin != nullptr && a.T >= 32 && !skip;
    int acc_p = -1;
    float acc_m = __int_as_float(0x7f800000);
    // the operands that do not depend on the accumulator -- this row's norm
    // and the running minimum and skip distance of every particle in the
    // warp's 128 columns -- loaded once per tile, before the first TMEM read
    // (a running minimum read early is only larger: more segments stored)
    const int nh = n0 + h * 128, pbase = nh / a.T;
    const int nend = min(a.N, nh + 128);
    const bool hoist = a.T >= 32;
    TileOps<float> nrm;
    TileOps<float> xsv;
    TileOps<unsigned int> run;
#pragma unroll
    for (int i = 0; i < kTileParticles; ++i) {
        const int p = pbase + i;
        const bool in = hoist && p * a.T < nend;
        nrm.set(i, (in && !skip) ? a.norm[(size_t)p * a.M + m] : 0.f);
        run.set(i, (in && a.segmask) ? __ldcg(&a.ps[p].min_coarse) : 0xFFFFFFFFu);
        xsv.set(i, (in && a.segmask) ? __ldg(&a.ps[p].xs) : 0.f);
    }
    for (int c = 0; c < 4; ++c) {
        const int col = h * 128 + c * 32;
        const int nb = n0 + col;
        if (nb >= a.N) break;  // warp-uniform
        const int nvalid = min(32, a.N - nb);
        // rows whose segments of this chunk are stored (bit r = lane r's row)
        unsigned int lo_rows = 0xFFFFFFFFu, hi_rows = 0xFFFFFFFFu;
        int bnd_st = 32;
        const int p_lo = nb / a.T;
        float v[32];
        tmem_ld32(acc + ((uint32_t)(q * 32) << 16) + (uint32_t)col, v);
        if (a.T >= 32) {
            // at most two particles in these 32 columns: p_lo for jj < bnd
            const int bnd = (p_lo + 1) * a.T - nb;
            const int il = p_lo - pbase;
            const float n_lo = nrm.get(il), n_hi = nrm.get(il + 1);
            const float xs_lo = xsv.get(il), xs_hi = xsv.get(il + 1);
            const unsigned int run_lo = run.get(il), run_hi = run.get(il + 1);
            bnd_st = bnd;
            float min_lo = __int_as_float(0x7f800000), min_hi = min_lo;
#pragma unroll
            for (int jj = 0; jj < 32; ++jj) {
                float d = __int_as_float(0x7f800000);
                if (!skip && jj < nvalid) {
                    d = (jj < bnd ? n_lo : n_hi) - 2.f * v[jj];
                    if (jj < bnd)
                        min_lo = fminf(min_lo, d);
                    else
                        min_hi = fminf(min_hi, d);
                }
                v[jj] = d;
            }
            const bool two = bnd < nvalid;
            const unsigned int u_lo = warp_min_flush(min_lo, &a.ps[p_lo].min_coarse);
            const unsigned int u_hi = two ? warp_min_flush(min_hi, &a.ps[p_lo + 1].min_coarse) : 0xFFFFFFFFu;
            if (a.segmask) {
                const bool near_lo = min_lo <= near_cut(min(u_lo, run_lo), xs_lo);
                const bool near_hi = two && min_hi <= near_cut(min(u_hi, run_hi), xs_hi);
                lo_rows = __ballot_sync(0xffffffffu, near_lo);
                hi_rows = __ballot_sync(0xffffffffu, near_hi);
                if (near_lo)
                    atomicOr(&a.segmask[(size_t)p_lo * a.M + m], 1u << ((nb >> 5) - ((p_lo * a.T) >> 5)));
                if (near_hi) atomicOr(&a.segmask[(size_t)(p_lo + 1) * a.M + m], 1u);
            }
            if (lo_rows | hi_rows) {
#pragma unroll
                for (int jj = 0; jj < 32; ++jj) tb[lane * 33 + jj] = v[jj];
            }
            if (track_rows) {
                if (p_lo != acc_p) {
                    rowmin_flush(a, acc_p, m, acc_m);
                    acc_p = p_lo;
                    acc_m = min_lo;
                } else {
                    acc_m = fminf(acc_m, min_lo);
                }
                if (two) {
                    rowmin_flush(a, acc_p, m, acc_m);
                    acc_p = p_lo + 1;
                    acc_m = min_hi;
                }
            }
        } else {
            // short translation lists: one particle index per column
            int p = p_lo, t = nb - p_lo * a.T;
            float lmin = __int_as_float(0x7f800000);
#pragma unroll
            for (int jj = 0; jj < 32; ++jj) {
                float d = __int_as_float(0x7f800000);
                if (jj < nvalid) {
                    if (!skip) {
                        d = a.norm[(size_t)p * a.M + m] - 2.f * v[jj];
                        lmin = fminf(lmin, d);
                    }
                    if (++t == a.T || jj + 1 == nvalid) {
                        warp_min_flush(lmin, &a.ps[p].min_coarse);
                        lmin = __int_as_float(0x7f800000);
                        t = 0;
                        ++p;
                    }
                }
                tb[lane * 33 + jj] = d;
            }
        }
        __syncwarp();
        // lane = column: each store writes 32 consecutive translations
        // of one row; rows whose segment is not kept are not stored
        const int n = nb + lane;
        if ((lo_rows | hi_rows) && lane < nvalid) {
            const int pn = n / a.T, tn = n - pn * a.T;
            float *dst = a.out + (size_t)pn * a.M * a.T + tn;
            const int rows = min(32, a.M - (m0 + q * 32));
            const unsigned int my_rows = lane < bnd_st ? lo_rows : hi_rows;
#pragma unroll 8
            for (int r = 0; r < 32; ++r)
                if (r < rows && ((my_rows >> r) & 1u)) dst[(size_t)(m0 + q * 32 + r) * a.T] = tb[r * 33 + lane];
        }
        __syncwarp();
    }
    if (track_rows) rowmin_flush(a, acc_p, m, acc_m);
}

// Persistent warp-specialised CTA, one per SM, tiles tidx = blockIdx.x +
// i * gridDim.x in tile_mn order.  Warp 0 lane 0 streams the pre-packed
// operand tiles with cp.async.bulk into the stage ring (full barriers count
// the bytes); warp 1 lane 0 issues the MMAs into one of two TMEM
// accumulators (256 columns each) and commits each stage to its empty
// barrier and each finished tile to its accumulator's tfull barrier; warps
// 4..11 drain the other accumulator meanwhile (warp w reads TMEM lanes
// 32 (w & 3).. and columns 128 ((w - 4) >> 2)..) and release it on tempty.
//
// kNorm: the same pipeline on TF32 operands (kind::tf32, K tiles of 32) for
// the norm term N(r,p) = sum_k |P_r(k)|^2 w_p(k); the epilogue stores the
// accumulator as out[p][M] (T = 1).
template <bool kNorm>
__global__ void __launch_bounds__(THREADS, 1) k_tc_diff2(const TcArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t full[STAGES];
    __shared__ __align__(8) uint64_t empty[STAGES];
    __shared__ __align__(8) uint64_t tfull[2];
    __shared__ __align__(8) uint64_t tempty[2];
    __shared__ __align__(8) uint64_t done;
    __shared__ uint32_t tmem_slot;
    __shared__ int sfail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nk = a.ktiles;
    const int ntotal = a.mtiles * a.ntiles;
    volatile int *vfail = &sfail;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(smem_u32(&tfull[b]), 1);
            mbar_init(smem_u32(&tempty[b]), EPI_WARPS);
        }
        mbar_init(smem_u32(&done), 1);
        sfail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    const uint32_t sbase = smem_u32(smem);

    if (warp == 0 && lane == 0) {
        // producer: one running stage counter over all tiles of this CTA
        uint32_t g = 0;
        const uint64_t keep = policy_keep();
        for (int tidx = blockIdx.x; tidx < ntotal && !*vfail; tidx += gridDim.x) {
            int mt, nt;
            tile_mn(tidx, a.group_m, a.mtiles, a.ntiles, mt, nt);
            // norms: A holds [hi | lo] (2 nk/3 tiles per row tile), read in the
            // order hi(0) hi(0) hi(1) hi(1) ... lo(0) lo(1) ... so that the
            // second read of each hi tile follows the first (an L2 hit)
            const int nkb = nk / 3;
            const uint8_t *ab = a.Ablk + (size_t)mt * (kNorm ? 2 * nkb : nk) * A_BYTES;
            const uint8_t *yb = a.Yblk + (size_t)nt * nk * B_BYTES;
            for (int kt = 0; kt < nk; ++kt, ++g) {
                const int ka = kNorm ? (kt < 2 * nkb ? kt >> 1 : kt - nkb) : kt;
                const uint32_t s = g % STAGES;
                if (g >= STAGES && !mbar_wait(smem_u32(&empty[s]), ((g / STAGES) - 1) & 1u)) {
                    *vfail = 1;
                    break;
                }
                const uint32_t st = sbase + s * STAGE_BYTES;
                arrive_expect_tx(smem_u32(&full[s]), (uint32_t)STAGE_BYTES);
                if (a.keep_a)
                    bulk_g2s_hint(st, ab + (size_t)ka * A_BYTES, A_BYTES, smem_u32(&full[s]), keep);
                else
                    bulk_g2s(st, ab + (size_t)ka * A_BYTES, A_BYTES, smem_u32(&full[s]));
                bulk_g2s(st + A_BYTES, yb + (size_t)kt * B_BYTES, B_BYTES, smem_u32(&full[s]));
            }
        }
        // copies still in flight (after a failure the MMA issuer stops
        // consuming) land before the CTA may leave: wait (bounded) for the
        // last filled phase of each stage; immediate when all were consumed
        for (uint32_t q = g > (uint32_t)STAGES ? g - STAGES : 0u; q < g; ++q)
            if (!mbar_wait(smem_u32(&full[q % STAGES]), (q / STAGES) & 1u)) *vfail = 1;
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        const uint32_t idesc = kNorm ? make_idesc_tf32() : make_idesc();
        uint32_t g = 0, i = 0;
        for (int tidx = blockIdx.x; tidx < ntotal && !*vfail; tidx += gridDim.x, ++i) {
            const uint32_t b = i & 1u;
            if (i >= 2 && !mbar_wait(smem_u32(&tempty[b]), ((i >> 1) - 1) & 1u)) {
                *vfail = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t acc = tmem + b * (uint32_t)TN;
            bool ok = true;
            for (int kt = 0; kt < nk; ++kt, ++g) {
                const uint32_t s = g % STAGES;
                if (!mbar_wait(smem_u32(&full[s]), (g / STAGES) & 1u)) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t a0 = sbase + s * STAGE_BYTES, b0 = a0 + A_BYTES;
#pragma unroll
                for (int kk = 0; kk < TK / 16; ++kk) {
                    const uint64_t ad = make_desc(a0 + kk * 256, 128, 1024);
                    const uint64_t bd = make_desc(b0 + kk * 256, 128, 1024);
                    if (kNorm)
                        mma_tf32(acc, ad, bd, idesc, (kt | kk) != 0 ? 1u : 0u);
                    else
                        mma_bf16(acc, ad, bd, idesc, (kt | kk) != 0 ? 1u : 0u);
                }
                mma_commit(smem_u32(&empty[s]));
            }
            if (!ok) {
                *vfail = 1;
                break;
            }
            mma_commit(smem_u32(&tfull[b]));
        }
        // completion of every MMA issued above (also after a failure)
        mma_commit(smem_u32(&done));
    } else if (warp >= 4) {
        const int ew = warp - 4, q = warp & 3, h = ew >> 2;
        float *tb = reinterpret_cast<float *>(smem + STAGES * STAGE_BYTES) + ew * 32 * 33;
        uint32_t i = 0;
        for (int tidx = blockIdx.x; tidx < ntotal && !*vfail; tidx += gridDim.x, ++i) {
            int mt, nt;
            tile_mn(tidx, a.group_m, a.mtiles, a.ntiles, mt, nt);
            const uint32_t b = i & 1u;
            if (!mbar_wait(smem_u32(&tfull[b]), (i >> 1) & 1u)) {
                *vfail = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int m0 = mt * TM, n0 = nt * TN;
            const int m = m0 + q * 32 + lane;
            if (kNorm) {
                // lane = row m; for each column the 32 lanes store 32 consecutive m
                for (int c = 0; c < 4; ++c) {
                    const int col = h * 128 + c * 32, nb = n0 + col;
                    if (nb >= a.N) break;  // warp-uniform
                    float v[32];
                    tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + b * (uint32_t)TN + (uint32_t)col, v);
                    const int nvalid = min(32, a.N - nb);
                    if (m < a.M) {
#pragma unroll
                        for (int jj = 0; jj < 32; ++jj)
                            if (jj < nvalid) a.out[(size_t)(nb + jj) * a.M + m] = v[jj];
                    }
                }
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                __syncwarp();
                if (lane == 0)
                    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[b]))
                                 : "memory");
                continue;
            }
            drain_cross(a, tmem + b * (uint32_t)TN, m0, n0, q, h, lane, tb);
            // accumulator drained: hand it back to the MMA issuer
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[b]))
                             : "memory");
        }
    }
    __syncwarp();
    if (warp == 0) {
        // every MMA of this CTA has completed before its tensor memory is freed
        bool ok = true;
        if (lane == 0) ok = mbar_wait(smem_u32(&done), 0u);
        ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
        if (!ok && lane == 0) *vfail = 1;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0 && *vfail) atomicCAS(&g_tc_error, 0, 1);
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// ---- cross term on SM pairs (cta_group::2) ----------------------------------
// A cluster of two CTAs on a pair of SMs computes output tiles of 256
// orientations x 256 columns.  Each CTA streams its own 128 orientation rows
// (A tile 2 mp + rank) and one half of the tile's particle columns (Y rows
// 128 rank ..); the MMA issued by the even CTA (M = 256, N = 256, K = 16)
// reads both CTAs' shared memory and writes each CTA's 128 x 256 half of the
// accumulator into that CTA's tensor memory.  Per SM and K tile that is 32 KB
// of operands instead of 48 KB for the same MMA work.
//
// Synchronisation: both CTAs' tensor copies (cp.async.bulk.tensor with
// .cta_group::2, over 2D views of the packed operands) complete their
// bytes on the even CTA's full barrier, whose producer expects both CTAs'
// bytes; the even CTA's commits release both CTAs' stages (empty) and
// accumulators (tfull, done); the epilogue warps of both CTAs hand an
// accumulator back on the even CTA's tempty barrier (16 arrivals).  Every
// mbarrier wait is bounded; both CTAs meet at a cluster barrier after their
// last wait, before the tensor memory (allocated by both CTAs together) is
// freed.
constexpr int P_STAGES = 6;
constexpr int P_HALF_BYTES = (TN / 2) * TK * 2;        // 16 KB: 128 Y rows x 64 K
constexpr int P_STAGE_BYTES = A_BYTES + P_HALF_BYTES;  // 32 KB
constexpr int P_SMEM_BYTES = P_STAGES * P_STAGE_BYTES + TRANSPOSE_BYTES;
// tensor-map view of a packed operand: rows of 2 KB (256 elements of 8
// bytes, the widest box row; a tensor copy costs about 9 clocks per box row,
// so 256-byte rows made the copies, not the MMAs, the limit), boxes of 8 rows
constexpr int P_ROW_BYTES = 2048, P_BOX_ROWS = 8;
static_assert(A_BYTES == P_ROW_BYTES * P_BOX_ROWS && P_HALF_BYTES == P_ROW_BYTES * P_BOX_ROWS, "16 KB boxes");

__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

__device__ __forceinline__ uint32_t cluster_id() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
    return r;
}

__device__ __forceinline__ uint32_t cluster_count() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
    return r;
}

// Shared::cluster address of the variable at local shared address `local`
// in the CTA of cluster rank `rank`.
__device__ __forceinline__ uint32_t rank_addr(uint32_t local, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
    return r;
}

// Arrive on a barrier of either CTA of the cluster (default semantics:
// release at CTA scope; the TMEM reads it orders are complete, waited for by
// tcgen05.wait::ld).  The cluster-scope form blocked the arriving warp for
// ~1,700 clocks per arrival.
__device__ __forceinline__ void arrive_cluster(uint32_t cluster_addr) {
    asm volatile("mbarrier.arrive.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr) : "memory");
}

// Bounded wait that acquires at cluster scope (arrivals from the peer CTA).
__device__ __forceinline__ bool mbar_wait_cl(uint32_t bar, uint32_t parity) {
    for (unsigned int it = 0; it < kWaitLimit; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// One 16 KB box (64 rows of 256 bytes, starting at row `row`) of a packed
// operand into this CTA's shared memory at dst; its bytes complete on the
// barrier at shared::cluster address bar (the even CTA's).  x = 0 always.
__device__ __forceinline__ void tma_box_pair(uint32_t dst, const CUtensorMap *map, int row, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cta.global.tile.mbarrier::complete_tx::bytes.cta_group::2 [%0], [%1, {%2, "
        "%3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(row), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void mma_bf16_pair(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                              uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrive on the barrier at shared::cluster address bar (either CTA of the
// pair) when every pair MMA issued so far by this thread has completed.
__device__ __forceinline__ void mma_commit_pair(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Instruction descriptor, kind::f16, M = 256 over the pair, N = TN.
__host__ __device__ constexpr uint32_t make_idesc_pair() {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) | ((uint32_t)(2 * TM >> 4) << 24);
}

__global__ void __launch_bounds__(THREADS, 1)
    k_tc_pair(const TcArgs a, const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapY) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t full[P_STAGES];
    __shared__ __align__(8) uint64_t empty[P_STAGES];
    __shared__ __align__(8) uint64_t tfull[2];
    __shared__ __align__(8) uint64_t tempty[2];
    __shared__ __align__(8) uint64_t done;
    __shared__ uint32_t tmem_slot;
    __shared__ int sfail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t rank = cluster_rank();
    const int cid = (int)cluster_id(), ncl = (int)cluster_count();
    const int nk = a.ktiles;
    const int mpairs = (a.mtiles + 1) >> 1;  // the A table holds an even number of row tiles
    const int ntotal = mpairs * a.ntiles;
    const int gp = max(1, a.group_m >> 1);
    volatile int *vfail = &sfail;

    if (warp == 0) {
        // one warp of each CTA of the pair allocates (the same columns in both)
        asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < P_STAGES; ++s) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(smem_u32(&tfull[b]), 1);
            mbar_init(smem_u32(&tempty[b]), 2 * EPI_WARPS);
        }
        mbar_init(smem_u32(&done), 1);
        sfail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    // both CTAs' barriers are initialised before either CTA signals the other
    cluster_sync_all();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    const uint32_t sbase = smem_u32(smem);

    if (warp == 0 && lane == 0) {
        // producer (both CTAs): this CTA's A rows and Y half of every stage,
        // completing on the even CTA's full barrier
        uint32_t g = 0;
        const uint32_t lead_full = rank_addr(smem_u32(&full[0]), 0);
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapA)) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapY)) : "memory");
        for (int tidx = cid; tidx < ntotal && !*vfail; tidx += ncl) {
            int mp, nt;
            tile_mn(tidx, gp, mpairs, a.ntiles, mp, nt);
            const int rowA = (2 * mp + (int)rank) * nk * P_BOX_ROWS;
            const int rowY = nt * nk * (2 * P_BOX_ROWS) + (int)rank * P_BOX_ROWS;
            for (int kt = 0; kt < nk; ++kt, ++g) {
                const uint32_t s = g % P_STAGES;
                if (g >= P_STAGES && !mbar_wait(smem_u32(&empty[s]), ((g / P_STAGES) - 1) & 1u)) {
                    *vfail = 1;
                    break;
                }
                const uint32_t st = sbase + s * P_STAGE_BYTES;
                // the even CTA's arrival announces both CTAs' bytes (the odd
                // CTA's may land first)
                if (rank == 0) arrive_expect_tx(smem_u32(&full[s]), 2u * P_STAGE_BYTES);
                tma_box_pair(st, &mapA, rowA + kt * P_BOX_ROWS, lead_full + s * 8u);
                tma_box_pair(st + A_BYTES, &mapY, rowY + kt * (2 * P_BOX_ROWS), lead_full + s * 8u);
            }
        }
        // the even CTA waits (bounded) for the last filled phase of each stage:
        // every copy of both CTAs that it announced has landed
        if (rank == 0)
            for (uint32_t q = g > (uint32_t)P_STAGES ? g - P_STAGES : 0u; q < g; ++q)
                if (!mbar_wait(smem_u32(&full[q % P_STAGES]), (q / P_STAGES) & 1u)) *vfail = 1;
    } else if (warp == 1 && lane == 0 && rank == 0) {
        // MMA issuer (even CTA)
        const uint32_t idesc = make_idesc_pair();
        uint32_t g = 0, i = 0;
        for (int tidx = cid; tidx < ntotal && !*vfail; tidx += ncl, ++i) {
            const uint32_t b = i & 1u;
            if (i >= 2 && !mbar_wait_cl(smem_u32(&tempty[b]), ((i >> 1) - 1) & 1u)) {
                *vfail = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t acc = tmem + b * (uint32_t)TN;
            bool ok = true;
            for (int kt = 0; kt < nk; ++kt, ++g) {
                const uint32_t s = g % P_STAGES;
                if (!mbar_wait(smem_u32(&full[s]), (g / P_STAGES) & 1u)) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t a0 = sbase + s * P_STAGE_BYTES, b0 = a0 + A_BYTES;
#pragma unroll
                for (int kk = 0; kk < TK / 16; ++kk) {
                    const uint64_t ad = make_desc(a0 + kk * 256, 128, 1024);
                    const uint64_t bd = make_desc(b0 + kk * 256, 128, 1024);
                    mma_bf16_pair(acc, ad, bd, idesc, (kt | kk) != 0 ? 1u : 0u);
                }
                mma_commit_pair(smem_u32(&empty[s]));
                mma_commit_pair(rank_addr(smem_u32(&empty[s]), 1));
            }
            if (!ok) {
                *vfail = 1;
                break;
            }
            mma_commit_pair(smem_u32(&tfull[b]));
            mma_commit_pair(rank_addr(smem_u32(&tfull[b]), 1));
        }
        // completion of every MMA issued above, in both CTAs (also after a failure)
        mma_commit_pair(smem_u32(&done));
        mma_commit_pair(rank_addr(smem_u32(&done), 1));
    } else if (warp >= 4) {
        const int ew = warp - 4, q = warp & 3, h = ew >> 2;
        float *tb = reinterpret_cast<float *>(smem + P_STAGES * P_STAGE_BYTES) + ew * 32 * 33;
        uint32_t i = 0;
        for (int tidx = cid; tidx < ntotal && !*vfail; tidx += ncl, ++i) {
            int mp, nt;
            tile_mn(tidx, gp, mpairs, a.ntiles, mp, nt);
            const uint32_t b = i & 1u;
            if (!mbar_wait(smem_u32(&tfull[b]), (i >> 1) & 1u)) {
                *vfail = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            drain_cross(a, tmem + b * (uint32_t)TN, (2 * mp + (int)rank) * TM, nt * TN, q, h, lane, tb);
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) arrive_cluster(rank_addr(smem_u32(&tempty[b]), 0));
        }
    }
    __syncwarp();
    if (warp == 0) {
        // every MMA writing this CTA's tensor memory has completed
        bool ok = true;
        if (lane == 0) ok = mbar_wait(smem_u32(&done), 0u);
        ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
        if (!ok && lane == 0) *vfail = 1;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    // neither CTA leaves (or frees its tensor memory) while the other may
    // still signal it or read its shared memory
    cluster_sync_all();
    if (tid == 0 && *vfail) atomicCAS(&g_tc_error, 0, 1);
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// A operand tiles: BF16 rows of the FP32 projection table, blocked per
// (M tile, K tile) in the no-swizzle K-major shared-memory image.
__global__ void k_pack_a(const float *__restrict__ src, int lds, int M, int K2, int ktiles, uint8_t *__restrict__ dst,
                         long long nchunks) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nchunks) return;
    const long long blk = c >> 10;  // 1024 chunks per A block
    const int within = (int)(c & 1023), row = within >> 3, kg = within & 7;
    const int mt = (int)(blk / ktiles), kt = (int)(blk - (long long)mt * ktiles);
    const int m = mt * TM + row, k0 = kt * TK + kg * 8;
    float f[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) f[i] = (m < M && k0 + i < K2) ? src[(size_t)m * lds + k0 + i] : 0.f;
    *reinterpret_cast<uint4 *>(dst + blk * A_BYTES + chunk_off(row, kg)) =
        make_uint4(pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), pack_bf16(f[4], f[5]), pack_bf16(f[6], f[7]));
}

// Eight BF16-bound values Y[(p,t)][8 kg .. 8 kg + 7] of K tile kt:
// Re/Im(b[p][j] E[t][j]) for the four pixels j of the chunk (zeros beyond npix).
__device__ __forceinline__ void y_chunk(const float2 *__restrict__ b, int ldb, const float2 *__restrict__ E,
                                        int lde, int npix, int p, int t, int kt, int kg, float (&y)[8]) {
    {
        const int j = kt * (TK / 2) + kg * 4;
        if (j + 4 <= ldb && j + 4 <= lde) {
            // rows padded to 16 pixels: two 16-byte loads each (zeros beyond npix)
            const float4 *bp = reinterpret_cast<const float4 *>(b + (size_t)p * ldb + j);
            const float4 *ep = reinterpret_cast<const float4 *>(E + (size_t)t * lde + j);
            const float4 x0 = __ldg(bp), x1 = __ldg(bp + 1), e0 = __ldg(ep), e1 = __ldg(ep + 1);
            const float xr[4] = {x0.x, x0.z, x1.x, x1.z}, xi[4] = {x0.y, x0.w, x1.y, x1.w};
            const float er[4] = {e0.x, e0.z, e1.x, e1.z}, ei[4] = {e0.y, e0.w, e1.y, e1.w};
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (j + q < npix) {
                    y[2 * q] = xr[q] * er[q] - xi[q] * ei[q];
                    y[2 * q + 1] = xr[q] * ei[q] + xi[q] * er[q];
                }
        } else {
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (j + q < npix) {
                    const float2 x = __ldg(b + (size_t)p * ldb + j + q), e = __ldg(E + (size_t)t * lde + j + q);
                    y[2 * q] = x.x * e.x - x.y * e.y;
                    y[2 * q + 1] = x.x * e.y + x.y * e.x;
                }
        }
    }
}

// B operand tiles: Y[(p,t)][2j+c] = Re/Im(b[p][j] E[t][j]) in BF16, blocked
// per (N tile, K tile) in the same image.
__global__ void k_pack_y(const float2 *__restrict__ b, int ldb, const float2 *__restrict__ E, int lde, int npix,
                         int T, int N, int ktiles, uint8_t *__restrict__ dst, long long nchunks) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nchunks) return;
    const long long blk = c >> 11;  // 2048 chunks per B block
    const int within = (int)(c & 2047), row = within >> 3, kg = within & 7;
    const int nt = (int)(blk / ktiles), kt = (int)(blk - (long long)nt * ktiles);
    const int n = nt * TN + row;
    float y[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) y[i] = 0.f;
    if (n < N) {
        const int p = n / T, t = n - p * T;
        y_chunk(b, ldb, E, lde, npix, p, t, kt, kg, y);
    }
    *reinterpret_cast<uint4 *>(dst + blk * B_BYTES + chunk_off(row, kg)) =
        make_uint4(pack_bf16(y[0], y[1]), pack_bf16(y[2], y[3]), pack_bf16(y[4], y[5]), pack_bf16(y[6], y[7]));
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t u;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(u) : "f"(x));
    return u;
}

// TF32 operand tiles of the norm term, three-term split (x = hi + lo, both
// rounded to TF32): one K loop of 3 nk tiles accumulates hi*hi and hi*lo
// for every K tile kt (steps 2 kt and 2 kt + 1), then lo*hi (steps 2 nk + kt).
// A (rows_t = 128) is stored [hi(0..nk-1) | lo(0..nk-1)]; B (rows_t = 256) in
// step order [hi(0) lo(0) hi(1) lo(1) ... | hi(0) hi(1) ...].  Tiles of
// rows_t rows by 32 values, same shared-memory image as the BF16 tiles
// (16-byte chunks of 4 values).
__global__ void k_pack_tf32(const float *__restrict__ src, int lds, int rows, int K, int nk, int rows_t, int is_b,
                            uint8_t *__restrict__ dst, long long nchunks) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nchunks) return;
    const int per = rows_t * 8;  // chunks per tile
    const long long blk = c / per;
    const int within = (int)(c - blk * per), row = within >> 3, kg = within & 7;
    const int ktot = (is_b ? 3 : 2) * nk;
    const int rt = (int)(blk / ktot), kk = (int)(blk - (long long)rt * ktot);
    int kt;
    bool lo;
    if (is_b) {
        lo = kk < 2 * nk && (kk & 1);
        kt = kk < 2 * nk ? kk >> 1 : kk - 2 * nk;
    } else {
        lo = kk >= nk;
        kt = lo ? kk - nk : kk;
    }
    const int r = rt * rows_t + row, k0 = kt * 32 + kg * 4;
    uint32_t u[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float x = (r < rows && k0 + i < K) ? src[(size_t)r * lds + k0 + i] : 0.f;
        const uint32_t hi = to_tf32(x);
        u[i] = lo ? to_tf32(x - __uint_as_float(hi)) : hi;
    }
    *reinterpret_cast<uint4 *>(dst + blk * (long long)(rows_t * 128) + chunk_off(row, kg)) =
        make_uint4(u[0], u[1], u[2], u[3]);
}

// ---- coarse pass restricted to orientation blocks -------------------------
// The same contraction with the roles of the operands exchanged, so that
// every particle can score its own set of orientations: the MMA's M axis is
// one particle's translations (T <= 128, rows beyond T zero) and its N axis
// one orientation block of NB consecutive rows of the projection table (the
// four sibling HEALPix directions of one parent pixel, every psi: NB = 4
// npsi).  A work item is one (particle, block) pair; the item list holds
// each particle's proposed blocks (all blocks for a particle that falls back
// to the exhaustive search), so restricted and exhaustive particles share
// one launch.  TMEM holds [translation][orientation]: for one accumulator
// column (an orientation row r) the 32 lanes of a warp are 32 consecutive
// translations, stored as one 128-byte segment of out[p][r][t].  Every
// scored row is stored whole, its row minimum recorded in rowmin and all of
// its 32-column segments marked in segmask; rows of blocks a particle did
// not score keep rowmin = ~0 and segmask = 0 (weight zero downstream).
constexpr int PB_MAX_N = 256;
constexpr int PB_A_BYTES = TM * TK * 2;                          // 16 KB: 128 translations x 64 K
constexpr int PB_STAGE_BYTES = PB_A_BYTES + PB_MAX_N * TK * 2;   // 48 KB
constexpr int PB_SMEM_BYTES = STAGES * PB_STAGE_BYTES;

struct TbArgs {
    const uint8_t *Yp;      // [nparticles][ktiles][PB_A_BYTES] per-particle Y tiles (rows = translations)
    const uint8_t *Bblk;    // [nblocks][ktiles][NB * 128] projection rows of each block
    const int2 *items;      // (particle, block) pairs
    int nitems, ktiles, NB, M, T;
    float *out;             // [p][M][T]
    const float *norm;      // [p][M]
    const float *pdf_orient;
    ParticleState *ps;
    unsigned int *rowmin;   // [p][M]
    unsigned int *segmask;  // [p][M]
};

__host__ __device__ constexpr uint32_t make_idesc_n(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Persistent CTA per SM over the item list (items blockIdx.x + i gridDim.x),
// with the warp roles, stage ring, double-buffered accumulators and bounded
// waits of k_tc_diff2.
__global__ void __launch_bounds__(THREADS, 1) k_tc_blocks(const TbArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t full[STAGES];
    __shared__ __align__(8) uint64_t empty[STAGES];
    __shared__ __align__(8) uint64_t tfull[2];
    __shared__ __align__(8) uint64_t tempty[2];
    __shared__ __align__(8) uint64_t done;
    __shared__ uint32_t tmem_slot;
    __shared__ int sfail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nk = a.ktiles;
    const uint32_t bbytes = (uint32_t)a.NB * (TK * 2);
    volatile int *vfail = &sfail;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(smem_u32(&tfull[b]), 1);
            mbar_init(smem_u32(&tempty[b]), EPI_WARPS);
        }
        mbar_init(smem_u32(&done), 1);
        sfail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    const uint32_t sbase = smem_u32(smem);

    if (warp == 0 && lane == 0) {
        uint32_t g = 0;
        for (int it = blockIdx.x; it < a.nitems && !*vfail; it += gridDim.x) {
            const int2 item = a.items[it];
            const uint8_t *yb = a.Yp + (size_t)item.x * nk * PB_A_BYTES;
            const uint8_t *bb = a.Bblk + (size_t)item.y * nk * bbytes;
            for (int kt = 0; kt < nk; ++kt, ++g) {
                const uint32_t s = g % STAGES;
                if (g >= STAGES && !mbar_wait(smem_u32(&empty[s]), ((g / STAGES) - 1) & 1u)) {
                    *vfail = 1;
                    break;
                }
                const uint32_t st = sbase + s * PB_STAGE_BYTES;
                arrive_expect_tx(smem_u32(&full[s]), (uint32_t)PB_A_BYTES + bbytes);
                bulk_g2s(st, yb + (size_t)kt * PB_A_BYTES, PB_A_BYTES, smem_u32(&full[s]));
                bulk_g2s(st + PB_A_BYTES, bb + (size_t)kt * bbytes, bbytes, smem_u32(&full[s]));
            }
        }
        for (uint32_t q = g > (uint32_t)STAGES ? g - STAGES : 0u; q < g; ++q)
            if (!mbar_wait(smem_u32(&full[q % STAGES]), (q / STAGES) & 1u)) *vfail = 1;
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = make_idesc_n(a.NB);
        uint32_t g = 0, i = 0;
        for (int it = blockIdx.x; it < a.nitems && !*vfail; it += gridDim.x, ++i) {
            const uint32_t b = i & 1u;
            if (i >= 2 && !mbar_wait(smem_u32(&tempty[b]), ((i >> 1) - 1) & 1u)) {
                *vfail = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t acc = tmem + b * (uint32_t)PB_MAX_N;
            bool ok = true;
            for (int kt = 0; kt < nk; ++kt, ++g) {
                const uint32_t s = g % STAGES;
                if (!mbar_wait(smem_u32(&full[s]), (g / STAGES) & 1u)) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t a0 = sbase + s * PB_STAGE_BYTES, b0 = a0 + PB_A_BYTES;
#pragma unroll
                for (int kk = 0; kk < TK / 16; ++kk) {
                    const uint64_t ad = make_desc(a0 + kk * 256, 128, 1024);
                    const uint64_t bd = make_desc(b0 + kk * 256, 128, 1024);
                    mma_bf16(acc, ad, bd, idesc, (kt | kk) != 0 ? 1u : 0u);
                }
                mma_commit(smem_u32(&empty[s]));
            }
            if (!ok) {
                *vfail = 1;
                break;
            }
            mma_commit(smem_u32(&tfull[b]));
        }
        mma_commit(smem_u32(&done));
    } else if (warp >= 4) {
        // warp (q, h): TMEM lanes 32 q.. (translations), columns h NB/2.. (rows)
        const int q = warp & 3, h = (warp - 4) >> 2;
        const int t = q * 32 + lane;
        const bool tv = t < a.T;
        const int half = a.NB >> 1;
        uint32_t i = 0;
        for (int it = blockIdx.x; it < a.nitems && !*vfail; it += gridDim.x, ++i) {
            const uint32_t b = i & 1u;
            if (!mbar_wait(smem_u32(&tfull[b]), (i >> 1) & 1u)) {
                *vfail = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int2 item = a.items[it];
            const int p = item.x;
            const size_t prow = (size_t)p * a.M;
            const int rbase = item.y * a.NB;
            // all 32-column segments of a row of particle p
            const int c0 = (p * a.T) >> 5, nch = ((p * a.T + a.T - 1) >> 5) - c0 + 1;
            const unsigned int segbits = nch >= 32 ? 0xFFFFFFFFu : ((1u << nch) - 1u);
            float pmin = __int_as_float(0x7f800000);
            for (int col = h * half; col < (h + 1) * half; col += 16) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + b * (uint32_t)PB_MAX_N + (uint32_t)col, v);
                unsigned int myrow = 0xFFFFFFFFu;
#pragma unroll
                for (int jj = 0; jj < 16; ++jj) {
                    const int r = rbase + col + jj;
                    const float pdf = __ldg(&a.pdf_orient[r]);
                    const float nrm = __ldg(&a.norm[prow + r]);
                    const float d = (tv && pdf > 0.f) ? nrm - 2.f * v[jj] : __int_as_float(0x7f800000);
                    if (tv) a.out[(prow + r) * a.T + t] = d;
                    pmin = fminf(pmin, d);
                    const unsigned int u = d < __int_as_float(0x7f800000) ? f2ord(d) : 0xFFFFFFFFu;
                    const unsigned int m = __reduce_min_sync(0xffffffffu, u);
                    if (lane == jj) myrow = m;
                }
                if (lane < 16) {
                    const size_t e = prow + rbase + col + lane;
                    if (myrow != 0xFFFFFFFFu) atomicMin(&a.rowmin[e], myrow);
                    if (q == 0) a.segmask[e] = segbits;
                }
            }
            warp_min_flush(pmin, &a.ps[p].min_coarse);
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[b]))
                             : "memory");
        }
    }
    __syncwarp();
    if (warp == 0) {
        bool ok = true;
        if (lane == 0) ok = mbar_wait(smem_u32(&done), 0u);
        ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
        if (!ok && lane == 0) *vfail = 1;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0 && *vfail) atomicCAS(&g_tc_error, 0, 1);
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// Per-particle Y tiles: rows = translations t < T of particle p (zero rows
// up to 128), [p][kt] tiles of PB_A_BYTES in the shared-memory image.
__global__ void k_pack_yp(const float2 *__restrict__ b, int ldb, const float2 *__restrict__ E, int lde, int npix,
                          int T, int ktiles, uint8_t *__restrict__ dst, long long nchunks) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nchunks) return;
    const long long blk = c >> 10;  // 1024 chunks per 128-row tile
    const int within = (int)(c & 1023), row = within >> 3, kg = within & 7;
    const int p = (int)(blk / ktiles), kt = (int)(blk - (long long)p * ktiles);
    float y[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) y[i] = 0.f;
    if (row < T) y_chunk(b, ldb, E, lde, npix, p, row, kt, kg, y);
    *reinterpret_cast<uint4 *>(dst + blk * PB_A_BYTES + chunk_off(row, kg)) =
        make_uint4(pack_bf16(y[0], y[1]), pack_bf16(y[2], y[3]), pack_bf16(y[4], y[5]), pack_bf16(y[6], y[7]));
}

// Projection rows in tiles of rows_t rows (one orientation block) x 64 K.
__global__ void k_pack_rows(const float *__restrict__ src, int lds, int M, int K2, int ktiles, int rows_t,
                            uint8_t *__restrict__ dst, long long nchunks) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nchunks) return;
    const int per = rows_t * 8;
    const long long blk = c / per;
    const int within = (int)(c - blk * per), row = within >> 3, kg = within & 7;
    const int mt = (int)(blk / ktiles), kt = (int)(blk - (long long)mt * ktiles);
    const int m = mt * rows_t + row, k0 = kt * TK + kg * 8;
    float f[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) f[i] = (m < M && k0 + i < K2) ? src[(size_t)m * lds + k0 + i] : 0.f;
    *reinterpret_cast<uint4 *>(dst + blk * (long long)(rows_t * TK * 2) + chunk_off(row, kg)) =
        make_uint4(pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), pack_bf16(f[4], f[5]), pack_bf16(f[6], f[7]));
}

}  // namespace

size_t tc_norm_a_bytes(int M, int K) { return (size_t)((M + TM - 1) / TM) * 2 * ((K + 31) / 32) * A_BYTES; }
size_t tc_norm_b_bytes(int N, int K) { return (size_t)((N + TN - 1) / TN) * 3 * ((K + 31) / 32) * B_BYTES; }

cudaError_t launch_tc_norm_pack_a(const float *src, int lds, int M, int K, void *dst, cudaStream_t st) {
    const int nk = (K + 31) / 32, mtiles = (M + TM - 1) / TM;
    const long long nchunks = (long long)mtiles * 2 * nk * (TM * 8);
    if (nchunks <= 0) return cudaSuccess;
    k_pack_tf32<<<(unsigned)((nchunks + 255) / 256), 256, 0, st>>>(src, lds, M, K, nk, TM, 0,
                                                                   static_cast<uint8_t *>(dst), nchunks);
    return cudaGetLastError();
}

// Row tiles of the packed projection table: an even count (the SM-pair
// kernel reads row tiles two at a time; a padding tile holds zeros).
static int a_row_tiles(int M) { return (((M + TM - 1) / TM) + 1) & ~1; }

size_t tc_a_bytes(int M, int K2) {
    return (size_t)a_row_tiles(M) * ((K2 + TK - 1) / TK) * A_BYTES;
}
size_t tc_y_bytes(int N, int K2) {
    return (size_t)((N + TN - 1) / TN) * ((K2 + TK - 1) / TK) * B_BYTES;
}

cudaError_t launch_tc_pack_a(const float *src, int lds, int M, int K2, void *dst, cudaStream_t st) {
    const int ktiles = (K2 + TK - 1) / TK, mtiles = a_row_tiles(M);
    const long long nchunks = (long long)mtiles * ktiles * (A_BYTES / 16);
    if (nchunks <= 0) return cudaSuccess;
    k_pack_a<<<(unsigned)((nchunks + 255) / 256), 256, 0, st>>>(src, lds, M, K2, ktiles, static_cast<uint8_t *>(dst),
                                                              nchunks);
    return cudaGetLastError();
}

// 2D view of a packed operand for tensor copies: rows of row_bytes bytes of
// 1-, 2- or 8-byte elements (elem), boxes of box_x elements x box_y rows.
static cudaError_t encode_view(const void *base, size_t bytes, int row_bytes, int elem, int box_x, int box_y,
                               CUtensorMap *out) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess) return e;
        if (!fn || q != cudaDriverEntryPointSuccess) return cudaErrorNotSupported;
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    if (((uintptr_t)base & 15u) != 0 || bytes % (size_t)row_bytes != 0 || (bytes / row_bytes) > 0x7fffffffULL)
        return cudaErrorInvalidValue;
    const cuuint64_t dims[2] = {(cuuint64_t)(row_bytes / elem), (cuuint64_t)(bytes / row_bytes)};
    const cuuint64_t strides[1] = {(cuuint64_t)row_bytes};
    const cuuint32_t box[2] = {(cuuint32_t)box_x, (cuuint32_t)box_y};
    const cuuint32_t estr[2] = {1, 1};
    if (elem != 1 && elem != 2 && elem != 8) return cudaErrorInvalidValue;
    const CUtensorMapDataType type = elem == 1   ? CU_TENSOR_MAP_DATA_TYPE_UINT8
                                     : elem == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT16
                                                 : CU_TENSOR_MAP_DATA_TYPE_UINT64;
    if (encode(out, type, 2,
               const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    return cudaSuccess;
}

cudaError_t launch_tc_diff2(const void *Ablk, void *Yblk, int M, int K2, const float2 *b, int ldb, const float2 *E,
                            int lde, int nparticles, int T, float *out, const float *norm, const float *pdf_orient,
                            ParticleState *ps, unsigned int *rowmin, unsigned int *segmask, cudaStream_t st,
                            const TcTuning &tune) {
    const int N = nparticles * T;
    if (N <= 0 || M <= 0) return cudaSuccess;
    const int ktiles = (K2 + TK - 1) / TK, ntiles = (N + TN - 1) / TN, mtiles = (M + TM - 1) / TM;
    const long long ychunks = (long long)ntiles * ktiles * (B_BYTES / 16);
    k_pack_y<<<(unsigned)((ychunks + 255) / 256), 256, 0, st>>>(b, ldb, E, lde, K2 / 2, T, N, ktiles,
                                                             static_cast<uint8_t *>(Yblk), ychunks);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const size_t smem = (size_t)SMEM_BYTES;
    static int nsm = 0;
    if (!nsm) {
        int dev = 0;
        e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_tc_diff2<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_tc_diff2<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) {
            nsm = 0;
            return e;
        }
    }
    const long long ntotal = (long long)mtiles * ntiles;
    if (ntotal > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    TcArgs a{static_cast<const uint8_t *>(Ablk), static_cast<const uint8_t *>(Yblk), M, ktiles, T, N, nparticles,
             mtiles, ntiles, out, norm, pdf_orient, ps, T >= 32 ? rowmin : nullptr,
             (T >= 32 && T <= 960 && rowmin) ? segmask : nullptr,
             tune.group_m > 0 ? tune.group_m : kGroupMDefault, tune.keep_a ? 1 : 0};
    if (tune.pair) {
        // 2D byte views of the packed operands for the tensor copies
        CUtensorMap maps[2];
        const size_t bytes[2] = {tc_a_bytes(M, K2), tc_y_bytes(N, K2)};
        e = encode_view(Ablk, bytes[0], P_ROW_BYTES, 8, P_ROW_BYTES / 8, P_BOX_ROWS, &maps[0]);
        if (e == cudaSuccess) e = encode_view(Yblk, bytes[1], P_ROW_BYTES, 8, P_ROW_BYTES / 8, P_BOX_ROWS, &maps[1]);
        if (e != cudaSuccess) return e;
        // clusters of two CTAs, as many as can be resident at once
        static int max_clusters = 0;
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = 2;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.blockDim = dim3(THREADS);
        cfg.dynamicSmemBytes = P_SMEM_BYTES;
        cfg.stream = st;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        if (!max_clusters) {
            e = cudaFuncSetAttribute(k_tc_pair, cudaFuncAttributeMaxDynamicSharedMemorySize, P_SMEM_BYTES);
            cfg.gridDim = dim3(2 * (unsigned)(nsm / 2));
            if (e == cudaSuccess) e = cudaOccupancyMaxActiveClusters(&max_clusters, k_tc_pair, &cfg);
            if (e != cudaSuccess) {
                max_clusters = 0;
                return e;
            }
            if (max_clusters <= 0) return cudaErrorInvalidConfiguration;
        }
        const long long npairs = (long long)((mtiles + 1) / 2) * ntiles;
        cfg.gridDim = dim3(2 * (unsigned)std::min<long long>(npairs, max_clusters));
        e = cudaLaunchKernelEx(&cfg, k_tc_pair, a, maps[0], maps[1]);
        if (e != cudaSuccess) return e;
        return cudaGetLastError();
    }
    const int grid = (int)std::min<long long>(ntotal, nsm);
    k_tc_diff2<false><<<grid, THREADS, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_tc_norm(const void *Ablk, const float *w, int ldw, int M, int K, int nparticles, void *Bblk,
                           float *out, cudaStream_t st) {
    if (nparticles <= 0 || M <= 0) return cudaSuccess;
    const int nk = (K + 31) / 32, ntiles = (nparticles + TN - 1) / TN, mtiles = (M + TM - 1) / TM;
    const long long bchunks = (long long)ntiles * 3 * nk * (TN * 8);
    k_pack_tf32<<<(unsigned)((bchunks + 255) / 256), 256, 0, st>>>(w, ldw, nparticles, K, nk, TN, 1,
                                                                   static_cast<uint8_t *>(Bblk), bchunks);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    static int nsm = 0;
    if (!nsm) {
        int dev = 0;
        e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_tc_diff2<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        if (e != cudaSuccess) {
            nsm = 0;
            return e;
        }
    }
    const long long ntotal = (long long)mtiles * ntiles;
    const int grid = (int)std::min<long long>(ntotal, nsm);
    TcArgs a{static_cast<const uint8_t *>(Ablk), static_cast<const uint8_t *>(Bblk), M, 3 * nk, 1, nparticles,
             nparticles, mtiles, ntiles, out, nullptr, nullptr, nullptr, nullptr, nullptr, kGroupMDefault, 0};
    k_tc_diff2<true><<<grid, THREADS, SMEM_BYTES, st>>>(a);
    return cudaGetLastError();
}

// ---- orientation-block restricted coarse pass ------------------------------
size_t tc_blocks_bytes(int M, int K2, int NB) {
    return (size_t)((M + NB - 1) / NB) * ((K2 + TK - 1) / TK) * (size_t)NB * TK * 2;
}
size_t tc_yp_bytes(int nparticles, int K2) { return (size_t)nparticles * ((K2 + TK - 1) / TK) * PB_A_BYTES; }

cudaError_t launch_tc_pack_blocks(const float *src, int lds, int M, int K2, int NB, void *dst, cudaStream_t st) {
    if (NB < 32 || NB > PB_MAX_N || NB % 32 != 0) return cudaErrorInvalidValue;
    const int ktiles = (K2 + TK - 1) / TK, nblk = (M + NB - 1) / NB;
    const long long nchunks = (long long)nblk * ktiles * NB * 8;
    if (nchunks <= 0) return cudaSuccess;
    k_pack_rows<<<(unsigned)((nchunks + 255) / 256), 256, 0, st>>>(src, lds, M, K2, ktiles, NB,
                                                                  static_cast<uint8_t *>(dst), nchunks);
    return cudaGetLastError();
}

cudaError_t launch_tc_blocks(const void *Bblk, int NB, void *Yp, int M, int K2, const float2 *b, int ldb,
                             const float2 *E, int lde, int nparticles, int T, const int2 *items, int nitems,
                             float *out, const float *norm, const float *pdf_orient, ParticleState *ps,
                             unsigned int *rowmin, unsigned int *segmask, cudaStream_t st) {
    if (nitems <= 0 || nparticles <= 0 || M <= 0) return cudaSuccess;
    if (T < 1 || T > TM || NB < 32 || NB > PB_MAX_N || NB % 32 != 0 || M % NB != 0 || !rowmin || !segmask)
        return cudaErrorInvalidValue;
    const int ktiles = (K2 + TK - 1) / TK;
    const long long ychunks = (long long)nparticles * ktiles * (PB_A_BYTES / 16);
    k_pack_yp<<<(unsigned)((ychunks + 255) / 256), 256, 0, st>>>(b, ldb, E, lde, K2 / 2, T, ktiles,
                                                                static_cast<uint8_t *>(Yp), ychunks);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    static int nsm = 0;
    if (!nsm) {
        int dev = 0;
        e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_tc_blocks, cudaFuncAttributeMaxDynamicSharedMemorySize, PB_SMEM_BYTES);
        if (e != cudaSuccess) {
            nsm = 0;
            return e;
        }
    }
    const int grid = std::min(nitems, nsm);
    TbArgs a{static_cast<const uint8_t *>(Yp), static_cast<const uint8_t *>(Bblk), items, nitems, ktiles, NB, M, T,
             out, norm, pdf_orient, ps, rowmin, segmask};
    k_tc_blocks<<<grid, THREADS, PB_SMEM_BYTES, st>>>(a);
    return cudaGetLastError();
}

// The same, queued on a stream: the flag is copied into page-locked host
// memory (valid after the caller's next synchronisation) and cleared.  No
// synchronous host-to-device copy: those wait behind any batch copy the
// host-to-device engine is serving for another stream.
cudaError_t tc_error_flag_async(int *host_flag, cudaStream_t st) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_tc_error);
    if (e == cudaSuccess) e = cudaMemcpyAsync(host_flag, p, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(p, 0, sizeof(int), st);
    return e;
}

cudaError_t tc_error_flag(int *flag, int reset) {
    cudaError_t e = cudaMemcpyFromSymbol(flag, g_tc_error, sizeof(int));
    if (e == cudaSuccess && reset) {
        const int z = 0;
        e = cudaMemcpyToSymbol(g_tc_error, &z, sizeof(int));
    }
    return e;
}

}  // namespace gbr
