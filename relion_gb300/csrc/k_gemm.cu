// k_gemm.cu -- coarse-pass contractions of the plain (FP32) path.
//
// The coarse squared difference of src/ml_optimiser.cpp:7436-7442,
//   diff2(r,p,t) = Xi2/2 + sum_k m_k |C_pk P_rk - X_pk E_tk|^2,
// m_k = invsigma2_k / 2, E_tk = exp(-2 pi i k.t / N), is evaluated as
//   diff2 = c_p + N(r,p) - 2 Re sum_k P_rk conj(m_k C_pk X_pk E_tk)
// with c_p = Xi2/2 + sum_k m_k |X_pk|^2 (per particle, FP64),
//      N(r,p) = sum_k (m_k C_pk^2) |P_rk|^2                (norm GEMM) and
// the cross term a real GEMM of K = 2 * active pixels (cross GEMM), whose
// B operand Y(p,t) = m C X E is formed on the fly while staging tiles, so
// it never exists in HBM.  The epilogue stores diff2 - c_p (relative to the
// per-particle constant, which cancels in every weight) in the reference's
// hidden-index order [p][r*T + t] and tracks the per-particle minimum.
//
// Tiles: 128x128 outputs per CTA, BK = 16, 256 threads with an 8x8
// register block each, double-buffered shared memory.
#include "gbr_internal.h"

namespace gbr {
namespace {

constexpr int BM = 128, BN = 128, BK = 16, NT = 256;

__device__ __forceinline__ unsigned int f2ord(float f) {
    unsigned int u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// B operand of the cross GEMM: Y[n][2j+c] = Re/Im(b[p][j] * E[t][j]).
struct CrossB {
    const float2 *b;   // [p][ldb]
    const float2 *E;   // [t][ldp]
    int ldb, ldp, T, N, npix;
    // Stage 8 consecutive k (4 pixels from pixel j) of column n.
    __device__ __forceinline__ void load(int n, int j, float v[8]) const {
        if (n >= N) {
#pragma unroll
            for (int i = 0; i < 8; ++i) v[i] = 0.f;
            return;
        }
        const int p = n / T, t = n - p * T;
        const float2 *bb = b + (size_t)p * ldb + j;
        const float2 *ee = E + (size_t)t * ldp + j;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            float2 x = make_float2(0.f, 0.f), e = make_float2(0.f, 0.f);
            if (j + i < npix) {
                x = __ldg(bb + i);
                e = __ldg(ee + i);
            }
            v[2 * i] = x.x * e.x - x.y * e.y;
            v[2 * i + 1] = x.x * e.y + x.y * e.x;
        }
    }
};

// B operand of the norm GEMM: plain rows a[n][k] (k contiguous, zero padded).
struct PlainB {
    const float *a;
    int lda, N;
    __device__ __forceinline__ void load(int n, int k8, float v[8]) const {
        if (n >= N) {
#pragma unroll
            for (int i = 0; i < 8; ++i) v[i] = 0.f;
            return;
        }
        const float4 *src = reinterpret_cast<const float4 *>(a + (size_t)n * lda + k8);
        float4 u0 = __ldg(src), u1 = __ldg(src + 1);
        v[0] = u0.x; v[1] = u0.y; v[2] = u0.z; v[3] = u0.w;
        v[4] = u1.x; v[5] = u1.y; v[6] = u1.z; v[7] = u1.w;
    }
};

template <bool kCross, class BL>
__global__ void __launch_bounds__(NT, 2)
k_gemm(const float *__restrict__ A, int lda, int M, int K, BL bl, int N, CrossEpilogue ep,
       float *__restrict__ out_norm) {
    __shared__ __align__(16) float As[2][BK][BM];
    __shared__ __align__(16) float Bs[2][BK][BN];
    __shared__ unsigned int smin[BN + 2];

    const int tid = threadIdx.x;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int lrow = tid & (BM - 1), lhalf = tid >> 7;  // loader: row/col, k half
    const int tm = tid >> 4, tn = tid & 15;               // compute: 4x4 groups

    if (kCross) {
        for (int i = tid; i < BN + 2; i += NT) smin[i] = 0xFFFFFFFFu;
    }

    float ra[8], rb[8];
    auto gload = [&](int k0) {
        const int m = m0 + lrow;
        if (m < M) {
            const float4 *src = reinterpret_cast<const float4 *>(A + (size_t)m * lda + k0 + lhalf * 8);
            float4 u0 = __ldg(src), u1 = __ldg(src + 1);
            ra[0] = u0.x; ra[1] = u0.y; ra[2] = u0.z; ra[3] = u0.w;
            ra[4] = u1.x; ra[5] = u1.y; ra[6] = u1.z; ra[7] = u1.w;
        } else {
#pragma unroll
            for (int i = 0; i < 8; ++i) ra[i] = 0.f;
        }
        if (kCross) bl.load(n0 + lrow, (k0 >> 1) + lhalf * 4, rb);
        else bl.load(n0 + lrow, k0 + lhalf * 8, rb);
    };
    auto sstore = [&](int buf) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            As[buf][lhalf * 8 + i][lrow] = ra[i];
            Bs[buf][lhalf * 8 + i][lrow] = rb[i];
        }
    };

    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;

    const int nk = (K + BK - 1) / BK;
    gload(0);
    sstore(0);
    __syncthreads();
    for (int kt = 0; kt < nk; ++kt) {
        const int cur = kt & 1;
        if (kt + 1 < nk) gload((kt + 1) * BK);
#pragma unroll
        for (int k = 0; k < BK; ++k) {
            float a[8], b[8];
            const float4 a0 = *reinterpret_cast<const float4 *>(&As[cur][k][tm * 4]);
            const float4 a1 = *reinterpret_cast<const float4 *>(&As[cur][k][64 + tm * 4]);
            const float4 b0 = *reinterpret_cast<const float4 *>(&Bs[cur][k][tn * 4]);
            const float4 b1 = *reinterpret_cast<const float4 *>(&Bs[cur][k][64 + tn * 4]);
            a[0] = a0.x; a[1] = a0.y; a[2] = a0.z; a[3] = a0.w;
            a[4] = a1.x; a[5] = a1.y; a[6] = a1.z; a[7] = a1.w;
            b[0] = b0.x; b[1] = b0.y; b[2] = b0.z; b[3] = b0.w;
            b[4] = b1.x; b[5] = b1.y; b[6] = b1.z; b[7] = b1.w;
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        if (kt + 1 < nk) {
            sstore(cur ^ 1);
            __syncthreads();
        }
    }

    // ---- epilogue ----
    if (kCross) {
        const int T = ep.T;
        const int p_first = n0 / T;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int m = m0 + (i < 4 ? tm * 4 + i : 64 + tm * 4 + (i - 4));
            if (m >= M) continue;
            const bool skip = !(ep.pdf_orient[m] > 0.f);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int n = n0 + (j < 4 ? tn * 4 + j : 64 + tn * 4 + (j - 4));
                if (n >= N) continue;
                const int p = n / T, t = n - p * T;
                float d;
                if (skip) {
                    d = __int_as_float(0x7f800000);  // +inf: not computed
                } else {
                    d = ep.norm[(size_t)p * M + m] - 2.f * acc[i][j];
                    atomicMin(&smin[p - p_first], f2ord(d));
                }
                ep.diff2[(size_t)p * ep.MT + (size_t)m * T + t] = d;
            }
        }
        __syncthreads();
        const int n_last = min(n0 + BN, N) - 1;
        const int np = n_last / T - p_first + 1;
        for (int i = tid; i < np; i += NT)
            if (smin[i] != 0xFFFFFFFFu) atomicMin(&ep.ps[p_first + i].min_coarse, smin[i]);
    } else {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int m = m0 + (i < 4 ? tm * 4 + i : 64 + tm * 4 + (i - 4));
            if (m >= M) continue;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int n = n0 + (j < 4 ? tn * 4 + j : 64 + tn * 4 + (j - 4));
                if (n < N) out_norm[(size_t)n * M + m] = acc[i][j];
            }
        }
    }
}

// Independent FMA chains per thread (8 accumulators) for a peak estimate.
__global__ void k_fp32_probe(float *out, int iters, float a, float b) {
    float x[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = threadIdx.x * 1e-3f + i;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) x[i] = fmaf(x[i], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += x[i];
    if (s == 12345.678f) out[0] = s;  // keep the chains live
}

}  // namespace

cudaError_t launch_fp32_probe(float *ms, double *flops) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    float *out = nullptr;
    cudaError_t e = cudaMalloc(&out, sizeof(float));
    if (e != cudaSuccess) return e;
    const int blocks = sms * 8, threads = 256, iters = 1 << 16;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    k_fp32_probe<<<blocks, threads>>>(out, 1024, 0.999f, 1e-3f);  // warm-up
    cudaEventRecord(a);
    k_fp32_probe<<<blocks, threads>>>(out, iters, 0.999f, 1e-3f);
    cudaEventRecord(b);
    e = cudaEventSynchronize(b);
    cudaEventElapsedTime(ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    *flops = 2.0 * 8.0 * (double)iters * blocks * threads;
    return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_gemm_cross(const float *A, int lda, int M, int K2, const float2 *bimg, int ldb,
                              const float2 *phase, int ldp, int nparticles, int T,
                              const CrossEpilogue &ep, cudaStream_t st) {
    const int N = nparticles * T;
    CrossB bl{bimg, phase, ldb, ldp, T, N, K2 / 2};
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
    if (grid.y > 65535) return cudaErrorInvalidConfiguration;
    k_gemm<true, CrossB><<<grid, NT, 0, st>>>(A, lda, M, K2, bl, N, ep, nullptr);
    return cudaGetLastError();
}

cudaError_t launch_gemm_norm(const float *A, int lda, int M, int K, const float *a, int lda_b,
                             int nparticles, float *out, cudaStream_t st) {
    PlainB bl{a, lda_b, nparticles};
    CrossEpilogue ep{};
    dim3 grid((nparticles + BN - 1) / BN, (M + BM - 1) / BM);
    k_gemm<false, PlainB><<<grid, NT, 0, st>>>(A, lda, M, K, bl, nparticles, ep, out);
    return cudaGetLastError();
}

}  // namespace gbr
