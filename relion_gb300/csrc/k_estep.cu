// k_estep.cu -- per-batch kernels of the E-step other than the coarse GEMMs:
// particle preparation, diff2 -> weight conversion, the significance
// threshold search, the fine (oversampled) pass, the weighted sums of
// storeWeightedSums and the Fourier backprojection.
//
// Reference semantics (CPU path, src/ml_optimiser.cpp):
//   weights      convertAllSquaredDifferencesToWeights  :7704-8239
//   significance sorted cumulative pruning              :8120-8200
//   fine pass    getAllSquaredDifferences (ipass 1)      :7098-7700
//   wsums / BP   storeWeightedSums                      :8241-9157
//   insertion    BackProjector::backproject2Dto3D        src/backprojector.cpp:55-296
#include "gbr_internal.h"

#include <algorithm>

#include <cfloat>

namespace gbr {
namespace {

__device__ __forceinline__ unsigned int f2ord(float f) {
    unsigned int u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned int u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide double sum; result valid in thread 0.  `sh` holds >= 32 doubles.
__device__ double block_sum(double v, double *sh) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double r = 0.;
    if (wid == 0) {
        r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.;
        r = warp_sum(r);
    }
    return r;
}

// ---------------------------------------------------------------------------
// Particle preparation: one block per particle.
//   coarse pixel j:  a_c = m C^2,  b_c = m C X          (m = invsigma2/2)
//   fine pixel j:    a_f, b_f likewise, plus compacted X, Xn, C
//   c = Xi2/2 + sum m |X|^2 in FP64 for each pass.
// pdat[p] = {old_x, old_y, prior_x, prior_y, highres_Xi2, norm, scale, 0}.
// ---------------------------------------------------------------------------
// Compensated (Kahan) FP32 summation: the sum's error stays near one FP32
// rounding of the total, whatever the number of terms, without FP64 adds
// (FP64 runs at a small fraction of the FP32 rate on this part).
__device__ __forceinline__ void kahan_add(float &s, float &c, float x) {
    const float y = x - c, t = s + y;
    c = (t - s) - y;
    s = t;
}

__global__ void k_prep(const float2 *__restrict__ X, const float *__restrict__ C,
                       const float2 *__restrict__ Xn, const double *__restrict__ pdat,
                       int full_npix, const PixelRef *__restrict__ pc, int nc,
                       const float *__restrict__ minv_c, int ldk_c, const PixelRef *__restrict__ pf,
                       int nf, int ldk_f, const float *__restrict__ minv_f, float *__restrict__ a_c,
                       float2 *__restrict__ b_c, float *__restrict__ a_f, float2 *__restrict__ b_f,
                       float2 *__restrict__ Xf, float2 *__restrict__ Xnf, float *__restrict__ Cf,
                       int do_scale, ParticleState *__restrict__ ps) {
    __shared__ double sh[32];
    const int p = blockIdx.x;
    const double *pd = pdat + (size_t)p * 8;
    const float scale = do_scale ? (float)pd[6] : 1.f;
    const float2 *x = X + (size_t)p * full_npix;
    const float2 *xn = Xn + (size_t)p * full_npix;
    const float *c = C + (size_t)p * full_npix;
    float ks = 0.f, kc = 0.f;  // sum of m |x|^2: FP32 terms, compensated FP32 per thread, FP64 across
    for (int j = threadIdx.x; j < ldk_c; j += blockDim.x) {
        float a = 0.f;
        float2 b = make_float2(0.f, 0.f);
        if (j < nc) {
            const int k = pc[j].full;
            const float cs = c[k] * scale, m = minv_c[j];
            const float2 v = x[k];
            a = m * cs * cs;
            b = make_float2(m * cs * v.x, m * cs * v.y);
            kahan_add(ks, kc, m * (v.x * v.x + v.y * v.y));
        }
        a_c[(size_t)p * ldk_c + j] = a;
        b_c[(size_t)p * ldk_c + j] = b;
    }
    double tot = block_sum((double)ks - (double)kc, sh);
    if (threadIdx.x == 0) {
        ParticleState s{};
        s.c_coarse = pd[4] / 2. + tot;
        s.min_coarse = 0xFFFFFFFFu;
        s.min_fine = 0xFFFFFFFFu;
        ps[p] = s;
    }
    ks = 0.f;
    kc = 0.f;
    for (int j = threadIdx.x; j < ldk_f; j += blockDim.x) {
        if (j >= nf) {
            a_f[(size_t)p * ldk_f + j] = 0.f;
            b_f[(size_t)p * ldk_f + j] = make_float2(0.f, 0.f);
            continue;
        }
        const int k = pf[j].full;
        const float cr = c[k];
        const float cs = cr * scale, m = minv_f[j];
        const float2 v = x[k];
        a_f[(size_t)p * ldk_f + j] = m * cs * cs;
        b_f[(size_t)p * ldk_f + j] = make_float2(m * cs * v.x, m * cs * v.y);
        Xf[(size_t)p * nf + j] = v;
        Xnf[(size_t)p * nf + j] = xn[k];
        Cf[(size_t)p * nf + j] = cr;
        kahan_add(ks, kc, m * (v.x * v.x + v.y * v.y));
    }
    tot = block_sum((double)ks - (double)kc, sh);
    if (threadIdx.x == 0) ps[p].c_fine = pd[4] / 2. + tot;
}

// pdf_offset per (particle, coarse translation), normalised by its mean over
// the translations (src/ml_optimiser.cpp:7779-7863, :7913-7958).  The
// translations tx, ty are in Angstrom and the old offset and prior in
// pixels, combined exactly as the reference does.
__global__ void k_pdf_offset(const double *__restrict__ pdat, const double *__restrict__ tx,
                             const double *__restrict__ ty, int T, double s2, double pixel,
                             float *__restrict__ out, double log_rt_orient, ParticleState *__restrict__ ps,
                             int KP, const double *__restrict__ class_prior) {
    __shared__ double sh[32];
    extern __shared__ double vals[];  // [KP][T]
    const int p = blockIdx.x;
    const double *pd = pdat + (size_t)p * 8;
    const int KT = KP * T;
    // The Gaussian's normalisation and any common factor cancel in the
    // normalisation by the mean below, so the exponent is taken relative to
    // its maximum over the particle's (class, translation) pairs, in FP32
    // (FP64 exponentials are slow on this GPU; the values are stored in FP32).
    double tmax = -DBL_MAX;
    const double neg_inv_2s2 = 1. / (-2. * s2);
    for (int i = threadIdx.x; i < KT; i += blockDim.x) {
        const int kc = i / T, t = i - kc * T;
        // 2D classification: the offset prior is the class's (:7829-7833)
        const double prx = class_prior ? class_prior[2 * kc] : pd[2];
        const double pry = class_prior ? class_prior[2 * kc + 1] : pd[3];
        const double ox = pd[0] + tx[t], oy = pd[1] + ty[t];
        // (x^2 + y^2) / (-2 s2) pixel^2, with one reciprocal per block
        const double td = ((ox - prx) * (ox - prx) + (oy - pry) * (oy - pry)) * neg_inv_2s2 * (pixel * pixel);
        vals[i] = td;
        tmax = fmax(tmax, td);
    }
    __shared__ double s_tmax;
    {
        for (int o = 16; o > 0; o >>= 1) tmax = fmax(tmax, __shfl_xor_sync(0xffffffffu, tmax, o));
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = tmax;
        __syncthreads();
        if (threadIdx.x == 0) {
            double m = -DBL_MAX;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, sh[w]);
            s_tmax = m;
        }
        __syncthreads();
    }
    double acc = 0.;
    for (int i = threadIdx.x; i < KT; i += blockDim.x) {
        const double td = vals[i];
        const double v = (s2 < 0.0001) ? ((td > 0.) ? 0. : 1.) : (double)expf((float)(td - s_tmax));
        vals[i] = v;
        acc += v;
    }
    double tot = block_sum(acc, sh);
    __shared__ double mean;
    if (threadIdx.x == 0) mean = tot / (double)KT;
    __syncthreads();
    float vmax = 0.f, vmin = FLT_MAX;
    const double inv_mean = mean > 0. ? 1. / mean : 1.;
    for (int i = threadIdx.x; i < KT; i += blockDim.x) {
        const float v = (float)(vals[i] * inv_mean);
        out[(size_t)p * KT + i] = v;
        vmax = fmaxf(vmax, v);
        vmin = fminf(vmin, v);
    }
    // Coarse skip distance: R T poses of weight at most pmax exp(-xs) stay
    // below 1e-10 pmin <= 1e-10 (largest weight) when
    // xs = ln(R T) + ln(pmax / pmin) + ln(1e10); log_rt_orient carries the
    // orientation part, +1 is margin for the FP32 exponential.
    __shared__ float smx[32], smn[32];
    for (int o = 16; o > 0; o >>= 1) {
        vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
        vmin = fminf(vmin, __shfl_xor_sync(0xffffffffu, vmin, o));
    }
    if ((threadIdx.x & 31) == 0) {
        smx[threadIdx.x >> 5] = vmax;
        smn[threadIdx.x >> 5] = vmin;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < (int)(blockDim.x >> 5); ++i) {
            vmax = fmaxf(vmax, smx[i]);
            vmin = fminf(vmin, smn[i]);
        }
        float xs = __int_as_float(0x7f800000);
        if (vmin > 0.f && vmax < FLT_MAX && isfinite(log_rt_orient))
            xs = (float)(log_rt_orient + log((double)vmax / (double)vmin) + 1.0);
        ps[p].xs = xs;
        ps[p].po_min = vmin;
    }
}

// ---------------------------------------------------------------------------
// diff2 -> weight, in place, over per-particle segments.  A block handles
// kChunk elements of one particle; also accumulates the FP64 weight sum, the
// level-0 histogram of the threshold search and (fine pass) the arg-max.
// ---------------------------------------------------------------------------
constexpr int kChunk = 8192;
constexpr int kWThreads = 512;
// k_weights_cand: orientation rows per block and loads in flight per lane
constexpr int kWRowsPerBlock = 2048;
constexpr int kWUnroll = 4;
constexpr int kCandBuf = 2048;  // block-local candidate buffer of k_weights_cand

__global__ void __launch_bounds__(kWThreads)
k_weights(float *__restrict__ vals, const long long *__restrict__ seg, int coarse, int T,
          const int *__restrict__ ejob, const unsigned int *__restrict__ ecode,
          const FineJob *__restrict__ jobs, int nOR, int nOT, const float *__restrict__ pdf_orient,
          const float *__restrict__ pdf_off, ParticleState *__restrict__ ps, int add_sum, int KP, int rpc,
          const unsigned int *__restrict__ segmask) {
    __shared__ double sh[32];
    __shared__ unsigned long long smax;
    const int p = blockIdx.y;
    const long long b0 = seg[p], b1 = seg[p + 1];
    const long long beg = b0 + (long long)blockIdx.x * kChunk;
    if (beg >= b1) return;
    const long long end = min(beg + (long long)kChunk, b1);
    if (threadIdx.x == 0) smax = 0ull;
    const float mn = ord2f(coarse == 1 ? ps[p].min_coarse : ps[p].min_fine);
    const float xcut = coarse == 1 ? fminf(ps[p].xs, 700.f) : 700.f;
    double acc = 0.;
    unsigned long long kmax = 0ull;
    const int Rrows = (int)((b1 - b0) / T);
    for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
        float d = vals[e];
        if (coarse == 1 && segmask) {
            // sparse coarse writes: a segment the coarse pass did not store
            // lies beyond the skip distance (weight 0)
            const unsigned int l32 = (unsigned int)(e - b0), rr = l32 / (unsigned int)T;
            const unsigned int tt = l32 - rr * (unsigned int)T;
            const unsigned int seg = segmask[(size_t)p * Rrows + rr];
            if (!((seg >> (((p * T + (int)tt) >> 5) - ((p * T) >> 5))) & 1u)) d = __int_as_float(0x7f800000);
        }
        float w = 0.f;
        if (d < FLT_MAX) {  // finite: computed
            const float x = d - mn;
            if (!(x > xcut)) {
                int r, t;
                unsigned int code = 0;
                const long long loc = e - b0;
                unsigned long long idx = 0;
                if (coarse == 1) {
                    const unsigned int l32 = (unsigned int)loc;  // < R*T < 2^32
                    r = (int)(l32 / (unsigned)T);
                    t = (int)(l32 - (unsigned)r * (unsigned)T);
                } else if (coarse == 2) {
                    // dense fine layout [rf][tf], rf = r*nOR + ior, tf = t*nOT + iot:
                    // the loop order of storeWeightedSums is the storage order
                    const long long TF = (long long)T * nOT;
                    r = (int)(loc / (TF * nOR));
                    t = (int)((loc % TF) / nOT);
                    idx = (unsigned long long)loc;
                } else {
                    r = jobs[ejob[e]].r;
                    code = ecode[e];
                    t = (int)(code / (unsigned)(nOR * nOT));
                    const unsigned int ior = (code / nOT) % nOR, iot = code % nOT;
                    idx = (((unsigned long long)r * nOR + ior) * T + t) * nOT + iot;
                }
                w = pdf_orient[r] * pdf_off[((size_t)p * KP + (KP > 1 ? r / rpc : 0)) * T + t] * expf(-x);
                if (coarse != 1 && w > 0.f) {
                    // loop order of storeWeightedSums: (r, iover_rot, itrans, iover_trans)
                    const unsigned long long key =
                        ((unsigned long long)__float_as_uint(w) << 32) | (0xFFFFFFFFull - idx);
                    kmax = key > kmax ? key : kmax;
                }
            }
        }
        vals[e] = w;
        acc += (double)w;
    }
    __syncthreads();
    const double tot = block_sum(acc, sh);
    if (coarse != 1) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long other = __shfl_xor_sync(0xffffffffu, kmax, o);
            kmax = other > kmax ? other : kmax;
        }
        if ((threadIdx.x & 31) == 0 && kmax) atomicMax(&smax, kmax);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (add_sum) atomicAdd(coarse == 1 ? &ps[p].sum_coarse : &ps[p].sum_fine, tot);
        if (coarse != 1 && smax) atomicMax(&ps[p].argmax_key, smax);
    }
}

// Coarse pass, first step: diff2 -> weight for every pose, FP64 sum, and a
// compact list of the candidates for significance: poses whose weight is at
// least eps_lo = (1 - fraction) * wmin / (R*T), where wmin (the smallest
// pdf_orient * pdf_offset) is a lower bound on the largest weight and hence
// eps_lo <= (1 - fraction) * sum / (R*T), the level below which no weight can
// reach the threshold.  Lists hold at most `cap` entries per particle
// (overflow -> flag; the driver then runs the full-array search).  The dense
// weight array is written only when `write_dense` is set.
__global__ void __launch_bounds__(kWThreads)
k_weights_cand(const float *__restrict__ vals, int R, int T, const float *__restrict__ pdf_orient,
               float pdf_orient_min, const float *__restrict__ pdf_off, double fraction,
               ParticleState *__restrict__ ps, unsigned int *__restrict__ cand_idx,
               float *__restrict__ cand_w, unsigned int *__restrict__ cand_cnt, int cap,
               float *__restrict__ dense_out, const unsigned int *__restrict__ rowmin, int KP, int rpc,
               const unsigned int *__restrict__ segmask, int cbuf, int rpb) {
    extern __shared__ float s_po[];  // pdf_offset rows of the classes of this block's orientations
    __shared__ double sh[32];
    __shared__ float s_eps;
    // candidates are gathered in a block-local buffer (shared-memory atomics)
    // and appended to the particle's list with one global atomic per flush
    __shared__ unsigned int s_ci[kCandBuf];
    __shared__ float s_cw[kCandBuf];
    __shared__ unsigned int s_n, s_cut;  // slots taken; first slot of an overflowing warp
    const int p = blockIdx.y;
    const int r0 = blockIdx.x * rpb;
    if (r0 >= R) return;
    if (threadIdx.x == 0) {
        s_n = 0u;
        s_cut = (unsigned)cbuf;
    }
    const int r1 = min(r0 + rpb, R);
    const long long RT = (long long)R * T;
    const int c0 = KP > 1 ? r0 / rpc : 0, c1 = KP > 1 ? (r1 - 1) / rpc : 0;
    for (int t = threadIdx.x; t < (c1 - c0 + 1) * T; t += blockDim.x)
        s_po[t] = pdf_off[((size_t)p * KP + c0) * T + t];
    if (threadIdx.x == 0)
        s_eps = (float)((1.0 - fraction) * (double)pdf_orient_min * (double)ps[p].po_min / (double)RT);
    __syncthreads();
    const float eps_lo = s_eps;
    const float mn = ord2f(ps[p].min_coarse);
    const float xs = fminf(ps[p].xs, 700.f);
    const float *rows = vals + (size_t)p * RT;
    unsigned int *ci = cand_idx + (size_t)p * cap;
    float *cw = cand_w + (size_t)p * cap;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    // candidates are summed in FP64; the rest (below eps_lo, together less
    // than (1 - fraction) of the total) in FP32, so the sum is FP64-accurate
    // to ~1e-10 relative without an FP64 add per pose
    double acc_c = 0.;
    float acc_f = 0.f;
    // Rows in batches of 32 per warp: each lane tests one row minimum, rows
    // beyond the skip distance are not read at all (the same float test as
    // for each pose: d >= rowmin gives d - mn >= rowmin - mn), and the warp
    // then walks the remaining rows in order, one warp per row so that
    // pdf_orient[r] is warp-uniform and the translation index is the lane.
    // each warp takes 4 x 32 rows per step: the four row-minimum loads of a
    // lane are issued together
    for (int rq = r0 + 128 * warp; rq < r1; rq += 128 * nwarps) {
    unsigned int ru4[4];
#pragma unroll
    for (int kq = 0; kq < 4; ++kq) {
        const int rr = rq + 32 * kq + lane;
        ru4[kq] = (rowmin && rr < r1) ? rowmin[(size_t)p * R + rr] : 0u;
    }
#pragma unroll
    for (int kq = 0; kq < 4; ++kq) {
        const int rb = rq + 32 * kq;
        const int rr = rb + lane;
        bool keep = rr < r1;
        if (keep && rowmin) {
            const unsigned int ru = ru4[kq];
            keep = !(ru == 0xFFFFFFFFu || ord2f(ru) - mn > xs);
            if (!keep && dense_out)
                for (int t = 0; t < T; ++t) dense_out[(size_t)p * RT + (size_t)rr * T + t] = 0.f;
        }
        unsigned int rows_left = __ballot_sync(0xffffffffu, keep);
        while (rows_left) {
            const int r = rb + __ffs(rows_left) - 1;
            rows_left &= rows_left - 1u;
            const float pr = pdf_orient[r];
            const float *po_r = s_po + (KP > 1 ? (r / rpc - c0) * T : 0);
            const float *row = rows + (size_t)r * T;
            // segments of the row the coarse pass stored (sparse writes); the
            // others lie beyond the skip distance and are not read
            const unsigned int seg = segmask ? segmask[(size_t)p * R + r] : 0xFFFFFFFFu;
            const int c0 = (p * T) >> 5;
            for (int t0 = 0; t0 < T; t0 += 32 * kWUnroll) {
                // kWUnroll independent streaming loads per lane, then one warp
                // vote: poses with diff2 - min > xs are skipped (all of them
                // together weigh less than 1e-10 of the sum)
                float dv[kWUnroll];
                bool near = false;
    #pragma unroll
                for (int k = 0; k < kWUnroll; ++k) {
                    const int t = t0 + 32 * k + lane;
                    const bool stored = t < T && ((seg >> (((p * T + t) >> 5) - c0)) & 1u);
                    dv[k] = stored ? __ldcs(row + t) : __int_as_float(0x7f800000);
                    near |= !(dv[k] - mn > xs);
                }
                if (!__any_sync(0xffffffffu, near)) {
                    if (dense_out) {
    #pragma unroll
                        for (int k = 0; k < kWUnroll; ++k) {
                            const int t = t0 + 32 * k + lane;
                            if (t < T) dense_out[(size_t)p * RT + (size_t)r * T + t] = 0.f;
                        }
                    }
                    continue;
                }
    #pragma unroll
                for (int k = 0; k < kWUnroll; ++k) {
                    const int t = t0 + 32 * k + lane;
                    float w = 0.f;
                    if (t < T) {
                        const float d = dv[k];
                        if (d < FLT_MAX) {
                            const float x = d - mn;
                            if (!(x > xs)) w = pr * po_r[t] * expf(-x);
                        }
                        if (dense_out) dense_out[(size_t)p * RT + (size_t)r * T + t] = w;
                    }
                    const bool is_c = w > 0.f && w >= eps_lo;
                    const unsigned int ball = __ballot_sync(0xffffffffu, is_c);
                    if (!is_c) acc_f += w;
                    if (ball) {  // warp-uniform: the FP64 add runs only where candidates are
                        if (is_c) acc_c += (double)w;
                        const unsigned int nb = (unsigned)__popc(ball);
                        unsigned int base = 0;
                        if (lane == 0) base = atomicAdd(&s_n, nb);
                        base = __shfl_sync(0xffffffffu, base, 0);
                        if (base + nb <= (unsigned)cbuf) {
                            if (is_c) {
                                const unsigned int pos = base + __popc(ball & ((1u << lane) - 1u));
                                s_ci[pos] = (unsigned int)((long long)r * T + t);
                                s_cw[pos] = w;
                            }
                        } else {
                            // buffer full: straight to the particle's list (the
                            // buffer keeps the slots below the first overflow)
                            if (lane == 0) atomicMin(&s_cut, base);
                            unsigned int gb = 0;
                            if (lane == 0) gb = atomicAdd(&cand_cnt[p], nb);
                            gb = __shfl_sync(0xffffffffu, gb, 0);
                            if (is_c) {
                                const unsigned int pos = gb + __popc(ball & ((1u << lane) - 1u));
                                if (pos < (unsigned)cap) {
                                    ci[pos] = (unsigned int)((long long)r * T + t);
                                    cw[pos] = w;
                                }
                            }
                        }
                    }
                }
            }
        }
    }
    }

    __syncthreads();
    {
        __shared__ unsigned int s_gbase;
        const unsigned int nbuf = min(s_n, s_cut);
        if (threadIdx.x == 0) s_gbase = nbuf ? atomicAdd(&cand_cnt[p], nbuf) : 0u;
        __syncthreads();
        for (unsigned int i = threadIdx.x; i < nbuf; i += blockDim.x) {
            const unsigned int pos = s_gbase + i;
            if (pos < (unsigned)cap) {
                ci[pos] = s_ci[i];
                cw[pos] = s_cw[i];
            }
        }
    }
    const double tot = block_sum(acc_c + (double)acc_f, sh);
    if (threadIdx.x == 0) atomicAdd(&ps[p].sum_coarse, tot);
}

// Significance masks and per-orientation counts from the candidate lists.
__global__ void k_cand_masks(const unsigned int *__restrict__ cand_idx, const float *__restrict__ cand_w,
                             const unsigned int *__restrict__ cand_cnt, int cap, int R, int T, int W,
                             const ParticleState *__restrict__ ps, unsigned int *__restrict__ mask,
                             int *__restrict__ cnt) {
    const int p = blockIdx.y;
    const unsigned int n = min(cand_cnt[p], (unsigned)cap);
    const float thr = ps[p].thr_coarse;
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float w = cand_w[(size_t)p * cap + i];
        if (w > 0.f && w >= thr) {
            const unsigned int e = cand_idx[(size_t)p * cap + i];
            const int r = (int)(e / (unsigned)T), t = (int)(e - (unsigned)r * (unsigned)T);
            atomicOr(&mask[((size_t)p * R + r) * W + (t >> 5)], 1u << (t & 31));
            atomicAdd(&cnt[(size_t)p * R + r], 1);
        }
    }
}

// Histogram of the threshold search: level 0 = top 12 bits of the weights;
// level 1 / 2 = the next 12 / 7 bits of the weights sharing the prefix
// selected so far.  With pass 1 / 2 (coarse / fine), weights below
// eps = (1 - fraction) * sum / (segment length) are skipped: the elements
// below eps sum to less than (1 - fraction) * sum, so the threshold is >= eps.
__global__ void __launch_bounds__(kWThreads)
k_hist_refine(const float *__restrict__ vals, const long long *__restrict__ seg, int level,
              const ParticleState *__restrict__ ps, HistBin *__restrict__ hist, int pass,
              double fraction, const long long *__restrict__ seg_end, long long n_total) {
    extern __shared__ double dsm[];
    double *hsum = dsm;
    unsigned int *hcnt = reinterpret_cast<unsigned int *>(hsum + kHistBins);
    const int p = blockIdx.y;
    const long long b0 = seg[p], b1 = seg_end ? seg_end[p] : seg[p + 1];
    const long long beg = b0 + (long long)blockIdx.x * kChunk;
    if (beg >= b1) return;
    const long long end = min(beg + (long long)kChunk, b1);
    const int nb = level == 2 ? 128 : kHistBins;
    const int shift = level == 0 ? 31 : (level == 1 ? 19 : 7);   // bits above the new field
    const int fshift = level == 0 ? 19 : (level == 1 ? 7 : 0);   // position of the new field
    const unsigned int fmask = level == 2 ? 0x7Fu : 0xFFFu;
    const unsigned int prefix = level == 0 ? 0u : ps[p].sel_prefix;
    float eps = 0.f;
    if (pass) {
        const double sum = pass == 1 ? ps[p].sum_coarse : ps[p].sum_fine;
        eps = (float)((1.0 - fraction) * sum / (double)(n_total > 0 ? n_total : b1 - b0));
    }
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        hsum[i] = 0.;
        hcnt[i] = 0u;
    }
    __syncthreads();
    for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
        const float w = vals[e];
        if (w > 0.f && w >= eps) {
            const unsigned int u = __float_as_uint(w);
            if ((u >> shift) == prefix) {
                const unsigned int bin = (u >> fshift) & fmask;
                atomicAdd(&hsum[bin], (double)w);
                atomicAdd(&hcnt[bin], 1u);
            }
        }
    }
    __syncthreads();
    HistBin *hp = hist + (size_t)p * kHistBins;
    for (int i = threadIdx.x; i < nb; i += blockDim.x)
        if (hcnt[i]) {
            atomicAdd(&hp[i].sum, hsum[i]);
            atomicAdd(&hp[i].count, hcnt[i]);
        }
}

// Histogram bins of the threshold search: in global memory (one HistBin per
// bin, filled by k_hist_refine) or in shared memory (k_select_fused).
struct GlobalBins {
    const HistBin *hp;
    __device__ double sum(int b) const { return hp[b].sum; }
    __device__ unsigned int count(int b) const { return hp[b].count; }
};
struct SharedBins {
    const double *hs;
    const unsigned int *hc;
    __device__ double sum(int b) const { return hs[b]; }
    __device__ unsigned int count(int b) const { return hc[b]; }
};

// Scratch of select_level in shared memory: one (sum, count) per thread.
struct SelectScratch {
    double *ssum;
    unsigned int *scnt;
    int *found_bin;
    double *found_above;
    unsigned int *found_cnt_above;
};

// One level of the search for the block's particle: walk the histogram from
// the largest weights down and find the bucket in which the cumulative
// weight first exceeds the target (the break of the loop at
// src/ml_optimiser.cpp:8158-8179).  After level 2 the bucket is a single
// float value: the significant weight.  All threads of the block take part.
template <class Bins>
__device__ void select_level(int level, double fraction, int coarse, ParticleState &s, const Bins &bins,
                             const SelectScratch &sc) {
    const int nb = level == 2 ? 128 : kHistBins;
    const int nt = (int)blockDim.x;
    const int per = (nb + nt - 1) / nt;   // bins per thread
    if (level == 0) {
        if (threadIdx.x == 0) {
            s.target = fraction * (coarse ? s.sum_coarse : s.sum_fine);
            s.sel_above = 0.;
            s.sel_count_above = 0u;
            s.sel_prefix = 0u;
        }
        __syncthreads();
    }
    const double target = s.target, above0 = s.sel_above;
    // thread i covers bins hi_i .. hi_i-per+1 (descending)
    const int hi = nb - 1 - (int)threadIdx.x * per;
    double my = 0.;
    unsigned int myc = 0;
    for (int q = 0; q < per; ++q) {
        const int b = hi - q;
        if (b >= 0) {
            my += bins.sum(b);
            myc += bins.count(b);
        }
    }
    sc.ssum[threadIdx.x] = my;
    sc.scnt[threadIdx.x] = myc;
    if (threadIdx.x == 0) *sc.found_bin = -1;
    __syncthreads();
    // inclusive scan (Hillis-Steele) over threads in descending-bin order
    for (int o = 1; o < nt; o <<= 1) {
        double v = threadIdx.x >= (unsigned)o ? sc.ssum[threadIdx.x - o] : 0.;
        unsigned int c = threadIdx.x >= (unsigned)o ? sc.scnt[threadIdx.x - o] : 0u;
        __syncthreads();
        sc.ssum[threadIdx.x] += v;
        sc.scnt[threadIdx.x] += c;
        __syncthreads();
    }
    const double incl = sc.ssum[threadIdx.x];
    const double excl = incl - my;
    const unsigned int excl_c = sc.scnt[threadIdx.x] - myc;
    if (above0 + excl <= target && above0 + incl > target) {
        double cum = above0 + excl;
        unsigned int cc = excl_c;
        for (int q = 0; q < per; ++q) {
            const int b = hi - q;
            if (b < 0) break;
            const double bs = bins.sum(b);
            if (cum + bs > target) {
                *sc.found_bin = b;
                *sc.found_above = cum;
                *sc.found_cnt_above = cc;
                break;
            }
            cum += bs;
            cc += bins.count(b);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && *sc.found_bin < 0) {
        // target not exceeded (fraction >= 1): the smallest positive weight
        double cum = above0;
        unsigned int cc = s.sel_count_above;
        int last = -1;
        for (int b = nb - 1; b >= 0; --b)
            if (bins.count(b)) {
                if (last >= 0) {
                    cum += bins.sum(last);
                    cc += bins.count(last);
                }
                last = b;
            }
        *sc.found_bin = last < 0 ? 0 : last;
        *sc.found_above = cum;
        *sc.found_cnt_above = cc - s.sel_count_above;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int b = *sc.found_bin;
        const unsigned int prefix = (level == 0) ? (unsigned)b
                                  : (level == 1) ? ((s.sel_prefix << 12) | (unsigned)b)
                                                 : ((s.sel_prefix << 7) | (unsigned)b);
        s.sel_prefix = prefix;
        s.sel_count_above += *sc.found_cnt_above;
        s.sel_above = *sc.found_above;
        if (level == 2) {
            const float v = __uint_as_float(prefix);
            // ties: the loop stops inside the run of equal values
            const double need = (s.target - s.sel_above) / (double)v;
            unsigned int k = (need >= 0.) ? (unsigned int)floor(need) + 1u : 1u;
            const unsigned int nb_cnt = bins.count(b);
            if (k > nb_cnt) k = nb_cnt;
            if (k < 1u) k = 1u;
            if (coarse) {
                s.thr_coarse = v;
                s.nr_sign = s.sel_count_above + k;
            } else {
                s.thr_fine = v;
            }
        }
    }
    __syncthreads();
}

// One block per particle, one level; the global histogram is cleared for
// the next level.
__global__ void k_select(int level, double fraction, int coarse, ParticleState *__restrict__ ps,
                         HistBin *__restrict__ hist) {
    __shared__ double ssum[256];
    __shared__ unsigned int scnt[256];
    __shared__ int found_bin;
    __shared__ double found_above;
    __shared__ unsigned int found_cnt_above;
    HistBin *hp = hist + (size_t)blockIdx.x * kHistBins;
    select_level(level, fraction, coarse, ps[blockIdx.x], GlobalBins{hp},
                 SelectScratch{ssum, scnt, &found_bin, &found_above, &found_cnt_above});
    for (int i = threadIdx.x; i < kHistBins; i += blockDim.x) {
        hp[i].sum = 0.;
        hp[i].count = 0u;
    }
}

// The whole three-level search of one particle in one block, histograms in
// shared memory: for segments short enough that one block streams them
// three times faster than six launches over many blocks (candidate lists,
// sparse fine entries).  Same filters and arithmetic as k_hist_refine +
// k_select.
constexpr int kSelThreads = 512;
__global__ void __launch_bounds__(kSelThreads)
k_select_fused(const float *__restrict__ vals, const long long *__restrict__ seg, const long long *__restrict__ seg_end,
               long long n_total, int pass, double fraction, int coarse, ParticleState *__restrict__ ps) {
    extern __shared__ double dsm[];
    double *hsum = dsm;
    double *ssum = hsum + kHistBins;
    unsigned int *hcnt = reinterpret_cast<unsigned int *>(ssum + kSelThreads);
    unsigned int *scnt = hcnt + kHistBins;
    __shared__ int found_bin;
    __shared__ double found_above;
    __shared__ unsigned int found_cnt_above;
    const int p = blockIdx.x;
    ParticleState &s = ps[p];
    const long long b0 = seg[p], b1 = seg_end ? seg_end[p] : seg[p + 1];
    float eps = 0.f;
    if (pass) {
        const double sum = pass == 1 ? s.sum_coarse : s.sum_fine;
        eps = (float)((1.0 - fraction) * sum / (double)(n_total > 0 ? n_total : b1 - b0));
    }
    const SelectScratch sc{ssum, scnt, &found_bin, &found_above, &found_cnt_above};
    for (int level = 0; level < 3; ++level) {
        const int nb = level == 2 ? 128 : kHistBins;
        const int shift = level == 0 ? 31 : (level == 1 ? 19 : 7);
        const int fshift = level == 0 ? 19 : (level == 1 ? 7 : 0);
        const unsigned int fmask = level == 2 ? 0x7Fu : 0xFFFu;
        for (int i = threadIdx.x; i < kHistBins; i += blockDim.x) {
            hsum[i] = 0.;
            hcnt[i] = 0u;
        }
        __syncthreads();
        const unsigned int prefix = level == 0 ? 0u : s.sel_prefix;
        for (long long e = b0 + threadIdx.x; e < b1; e += blockDim.x) {
            const float w = vals[e];
            if (w > 0.f && w >= eps) {
                const unsigned int u = __float_as_uint(w);
                if ((u >> shift) == prefix) {
                    const unsigned int bin = (u >> fshift) & fmask;
                    atomicAdd(&hsum[bin], (double)w);
                    atomicAdd(&hcnt[bin], 1u);
                }
            }
        }
        __syncthreads();
        (void)nb;
        select_level(level, fraction, coarse, s, SharedBins{hsum, hcnt}, sc);
    }
}

// Significance bitmask per (particle, coarse orientation): bit t set where
// the coarse weight >= the significant weight (Mcoarse_significant,
// src/ml_optimiser.cpp:8210-8218).  One warp per (p, r).
__global__ void k_sig_masks(const float *__restrict__ w, int n, int R, int T, int W,
                            const ParticleState *__restrict__ ps, unsigned int *__restrict__ mask,
                            int *__restrict__ cnt) {
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (gw >= (long long)n * R) return;
    const int p = (int)(gw / R);
    const float thr = ps[p].thr_coarse;
    const float *row = w + (size_t)gw * T;
    int c = 0;
    for (int word = 0; word < W; ++word) {
        const int t = word * 32 + lane;
        const float v = t < T ? row[t] : 0.f;
        const unsigned int bits = __ballot_sync(0xffffffffu, v > 0.f && v >= thr);
        if (lane == 0) mask[(size_t)gw * W + word] = bits;
        c += __popc(bits);
    }
    if (lane == 0) cnt[gw] = c;
}

// Exclusive scan of int64 (out has n+1 entries, out[n] = total).
constexpr int kScanBlock = 1024;
// Fine-pass job list in three launches (reduce, scan of the block sums,
// re-scan and emit), for the pairs (flag = cnt > 0, entries = cnt * per) of
// every (particle, coarse orientation) in (p, r) order.
__device__ __forceinline__ void block_excl_scan2(long long &a, long long &b, long long *wa, long long *wb,
                                                 long long &ta, long long &tb) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    long long ia = a, ib = b;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long xa = __shfl_up_sync(0xffffffffu, ia, o), xb = __shfl_up_sync(0xffffffffu, ib, o);
        if (lane >= o) {
            ia += xa;
            ib += xb;
        }
    }
    __syncthreads();
    if (lane == 31) {
        wa[warp] = ia;
        wb[warp] = ib;
    }
    __syncthreads();
    if (warp == 0) {
        const long long va = lane < nw ? wa[lane] : 0, vb = lane < nw ? wb[lane] : 0;
        long long sa = va, sb = vb;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long xa = __shfl_up_sync(0xffffffffu, sa, o), xb = __shfl_up_sync(0xffffffffu, sb, o);
            if (lane >= o) {
                sa += xa;
                sb += xb;
            }
        }
        const long long tot_a = __shfl_sync(0xffffffffu, sa, 31), tot_b = __shfl_sync(0xffffffffu, sb, 31);
        if (lane < nw) {
            wa[lane] = sa - va;
            wb[lane] = sb - vb;
        }
        if (lane == 0) {
            wa[32] = tot_a;
            wb[32] = tot_b;
        }
    }
    __syncthreads();
    a = ia - a + wa[warp];
    b = ib - b + wb[warp];
    ta = wa[32];
    tb = wb[32];
}

// Job-list kernels: each thread takes kJobsPer consecutive (particle,
// orientation) counts (vector loads; the array is mostly zeros), a block
// kJobsThreads * kJobsPer of them.
constexpr int kJobsThreads = 256, kJobsPer = 16;

__device__ __forceinline__ void load_counts(const int *__restrict__ cnt, long long base, long long tot,
                                            int (&c)[kJobsPer]) {
    if (base + kJobsPer <= tot && (base & 3) == 0) {
        const int4 *v = reinterpret_cast<const int4 *>(cnt + base);
#pragma unroll
        for (int q = 0; q < kJobsPer / 4; ++q) {
            const int4 x = __ldg(v + q);
            c[4 * q] = x.x;
            c[4 * q + 1] = x.y;
            c[4 * q + 2] = x.z;
            c[4 * q + 3] = x.w;
        }
    } else {
#pragma unroll
        for (int q = 0; q < kJobsPer; ++q) c[q] = (base + q < tot) ? cnt[base + q] : 0;
    }
}

__global__ void __launch_bounds__(kJobsThreads) k_jobs_reduce(const int *__restrict__ cnt, long long n, int per,
                                                             long long *__restrict__ sums) {
    __shared__ long long wa[33], wb[33];
    const long long base = ((long long)blockIdx.x * kJobsThreads + threadIdx.x) * kJobsPer;
    int c[kJobsPer];
    load_counts(cnt, base, n, c);
    long long f = 0, e = 0, tf, te;
#pragma unroll
    for (int q = 0; q < kJobsPer; ++q) {
        f += c[q] > 0 ? 1 : 0;
        e += (long long)c[q] * per;
    }
    block_excl_scan2(f, e, wa, wb, tf, te);
    if (threadIdx.x == 0) {
        sums[2 * blockIdx.x] = tf;
        sums[2 * blockIdx.x + 1] = te;
    }
}

// Exclusive scan of nb (flag, entries) block sums in place by one block;
// the totals land in sums[2 nb], sums[2 nb + 1].
__global__ void __launch_bounds__(kScanBlock) k_jobs_scan_sums(long long *__restrict__ sums, int nb) {
    __shared__ long long wa[33], wb[33];
    const int per_t = (nb + kScanBlock - 1) / kScanBlock;
    const int b0 = threadIdx.x * per_t, b1 = min(b0 + per_t, nb);
    long long f = 0, e = 0;
    for (int b = b0; b < b1; ++b) {
        f += sums[2 * b];
        e += sums[2 * b + 1];
    }
    long long tf, te;
    block_excl_scan2(f, e, wa, wb, tf, te);
    for (int b = b0; b < b1; ++b) {
        const long long vf = sums[2 * b], ve = sums[2 * b + 1];
        sums[2 * b] = f;
        sums[2 * b + 1] = e;
        f += vf;
        e += ve;
    }
    if (threadIdx.x == 0) {
        sums[2 * nb] = tf;
        sums[2 * nb + 1] = te;
    }
}

__global__ void __launch_bounds__(kJobsThreads) k_jobs_emit(const int *__restrict__ cnt, int n, int R, int per,
                                                           const long long *__restrict__ sums, int nb,
                                                           FineJob *__restrict__ jobs, long long *__restrict__ seg,
                                                           unsigned char *__restrict__ need_r) {
    __shared__ long long wa[33], wb[33];
    const long long tot = (long long)n * R;
    const long long base = ((long long)blockIdx.x * kJobsThreads + threadIdx.x) * kJobsPer;
    int c[kJobsPer];
    load_counts(cnt, base, tot, c);
    long long f = 0, e = 0, tf, te;
#pragma unroll
    for (int q = 0; q < kJobsPer; ++q) {
        f += c[q] > 0 ? 1 : 0;
        e += (long long)c[q] * per;
    }
    block_excl_scan2(f, e, wa, wb, tf, te);
    f += sums[2 * blockIdx.x];
    e += sums[2 * blockIdx.x + 1];
    if (base < tot) {
        int p = (int)(base / R), r = (int)(base - (long long)p * R);
        for (int q = 0; q < kJobsPer && base + q < tot; ++q) {
            if (r == 0) seg[p] = e;
            if (c[q] > 0) {
                FineJob j;
                j.p = p;
                j.r = r;
                j.n_t = c[q];
                j.pad_ = 0;
                j.off = e;
                jobs[f] = j;
                need_r[r] = 1;
                ++f;
                e += (long long)c[q] * per;
            }
            if (++r == R) {
                r = 0;
                ++p;
            }
        }
    }
    if (base == 0) seg[n] = sums[2 * nb + 1];
}

// ---------------------------------------------------------------------------
// Fine pass over a device work queue: a work item is one job (particle p,
// coarse orientation r) and one range of kFineSplit fine pixels; jobs with
// many significant translations and jobs with few share one persistent
// launch whose blocks take the next item from a device counter.  For every
// oversampled orientation ior and every significant coarse translation t
// with its oversampled shifts iot:
//   diff2 - c_fine = N_ior - 2 sum_k Re(Q_ior,k conj(E_(t,iot),k)),
//   Q = P_(r,ior) conj(m C X),  N_ior = sum_k m C^2 |P|^2.
// Q is staged in shared memory per chunk of kFineChunk pixels.  A warp takes
// kFineRows rows (t, iot) at a time: each Q value read from shared memory
// serves kFineRows rows, and the warp's 32 partial sums (kFineRows rows x 8
// orientations) are reduced across the lanes in one 31-shuffle
// transpose-reduction.  Each item stores its partial sums; the job's last
// item to finish (arrival counter) adds the partials in range order (the
// result does not depend on which block ran which range), writes the entries
// in hidden-index order (t, ior, iot) and the particle's minimum.
// ---------------------------------------------------------------------------
constexpr int kFineChunk = 512;
constexpr int kFineSplit = 2 * kFineChunk;  // fine pixels per work item
constexpr int kFineThreads = 256;
constexpr int kFineRows = 4;  // rows per warp pass; kFineRows x 8 orientations = 32 lanes

// v[i] summed over the warp's lanes, the sum of index i left on lane i
// (recursive halving: at offset o each lane keeps the half whose index bit
// equals its own lane bit and adds the partner's copy of it).
__device__ __forceinline__ float warp_transpose_sum32(float (&v)[32], int lane) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < o; ++i) {
            const float send = upper ? v[i] : v[i + o];
            const float keep = upper ? v[i + o] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    return v[0];
}

struct FineQueue {
    const long long *njobs;        // device: number of jobs
    int nsplit;                    // pixel ranges per job
    unsigned long long *head;      // next work item (zero at launch)
    int *arrive;                   // [njobs] items finished (zero at launch)
    float *part;                   // [nfine][nsplit] partial cross sums
    float *npart;                  // [njobs][8][nsplit] partial norms
};

__global__ void __launch_bounds__(kFineThreads, 4)
k_fine_diff2(const FineJob *__restrict__ jobs, const FineQueue qu, const unsigned int *__restrict__ mask, int R,
             int T, int W, int nOR, int nOT, const float2 *__restrict__ projf, int ldpf,
             const float2 *__restrict__ b_f, const float *__restrict__ a_f, int nf,
             const float2 *__restrict__ phase_f, float *__restrict__ d, int *__restrict__ ejob,
             unsigned int *__restrict__ ecode, ParticleState *__restrict__ ps) {
    extern __shared__ float4 fsm[];
    float2 *Q = reinterpret_cast<float2 *>(fsm);                   // [8][kFineChunk]
    float *acc = reinterpret_cast<float *>(Q + 8 * kFineChunk);    // [rows][nOR]
    int *tlist = reinterpret_cast<int *>(acc + T * nOT * nOR);     // [T]
    float *norm = reinterpret_cast<float *>(tlist + T);            // [nOR]
    __shared__ unsigned int smin;
    __shared__ unsigned long long item_s;
    __shared__ int last_s;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const int S = qu.nsplit;
    const unsigned long long total = (unsigned long long)(*qu.njobs) * (unsigned long long)S;
    // orientations nOR..7 of Q stay zero (their sums are not stored)
    for (int i = nOR * kFineChunk + threadIdx.x; i < 8 * kFineChunk; i += blockDim.x) Q[i] = make_float2(0.f, 0.f);
    for (;;) {
        if (threadIdx.x == 0) item_s = atomicAdd(qu.head, 1ull);
        __syncthreads();
        const unsigned long long item = item_s;
        if (item >= total) break;
        const long long jid = (long long)(item / (unsigned long long)S);
        const int sidx = (int)(item - (unsigned long long)jid * S);
        const FineJob job = jobs[jid];
        const int p = job.p, r = job.r, n_t = job.n_t;
        const int rows = n_t * nOT;
        if (threadIdx.x == 0) {
            const unsigned int *mk = mask + ((size_t)p * R + r) * W;
            int m = 0;
            for (int w = 0; w < W; ++w) {
                unsigned int bits = mk[w];
                while (bits) {
                    const int b = __ffs(bits) - 1;
                    bits &= bits - 1;
                    tlist[m++] = w * 32 + b;
                }
            }
            smin = 0xFFFFFFFFu;
        }
        for (int i = threadIdx.x; i < rows * nOR; i += blockDim.x) acc[i] = 0.f;
        for (int i = threadIdx.x; i < nOR; i += blockDim.x) norm[i] = 0.f;
        __syncthreads();
        const float2 *bp = b_f + (size_t)p * ldpf;
        const float *ap = a_f + (size_t)p * ldpf;
        const int kend = min(nf, (sidx + 1) * kFineSplit);
        for (int c0 = sidx * kFineSplit; c0 < kend; c0 += kFineChunk) {
            const int cl = min(kFineChunk, kend - c0);
            // stage Q, accumulate norms (one warp per ior at a time)
            for (int ior = warp; ior < nOR; ior += nwarp) {
                const float2 *P = projf + ((size_t)r * nOR + ior) * ldpf + c0;
                float nacc = 0.f;
                for (int k = lane; k < cl; k += 32) {
                    const float2 pv = P[k], bv = bp[c0 + k];
                    Q[ior * kFineChunk + k] = make_float2(pv.x * bv.x + pv.y * bv.y, pv.y * bv.x - pv.x * bv.y);
                    nacc = fmaf(ap[c0 + k], pv.x * pv.x + pv.y * pv.y, nacc);
                }
                nacc = warp_sum(nacc);
                if (lane == 0) norm[ior] += nacc;
            }
            __syncthreads();
            for (int row0 = warp * kFineRows; row0 < rows; row0 += nwarp * kFineRows) {
                const float2 *E[kFineRows];
#pragma unroll
                for (int j = 0; j < kFineRows; ++j) {
                    const int row = min(row0 + j, rows - 1);  // rows past the end repeat the last (not stored)
                    const int tr = row / nOT, iot = row - tr * nOT;
                    E[j] = phase_f + (size_t)(tlist[tr] * nOT + iot) * nf + c0;
                }
                float sacc[32];
#pragma unroll
                for (int i = 0; i < 32; ++i) sacc[i] = 0.f;
                for (int k = lane; k < cl; k += 32) {
                    float2 q[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) q[i] = Q[i * kFineChunk + k];
#pragma unroll
                    for (int j = 0; j < kFineRows; ++j) {
                        const float2 e = E[j][k];
#pragma unroll
                        for (int i = 0; i < 8; ++i)
                            sacc[j * 8 + i] = fmaf(q[i].x, e.x, fmaf(q[i].y, e.y, sacc[j * 8 + i]));
                    }
                }
                const float v = warp_transpose_sum32(sacc, lane);
                const int row = row0 + (lane >> 3), ior = lane & 7;
                if (row < rows && ior < nOR) acc[row * nOR + ior] += v;
            }
            __syncthreads();
        }
        // this range's partial sums; entry = off + (tr*nOR + ior)*nOT + iot
        for (int i = threadIdx.x; i < rows * nOR; i += blockDim.x) {
            const int row = i / nOR, ior = i - row * nOR;
            const int tr = row / nOT, iot = row - tr * nOT;
            const long long e = job.off + ((long long)tr * nOR + ior) * nOT + iot;
            qu.part[e * S + sidx] = acc[i];
        }
        for (int i = threadIdx.x; i < nOR; i += blockDim.x) qu.npart[((size_t)jid * 8 + i) * S + sidx] = norm[i];
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) last_s = atomicAdd(&qu.arrive[jid], 1) == S - 1;
        __syncthreads();
        if (last_s) {
            // the job's last range: sum the partials in range order
            __threadfence();
            if (threadIdx.x < nOR) {
                float nsum = 0.f;
                for (int q = 0; q < S; ++q) nsum += __ldcg(&qu.npart[((size_t)jid * 8 + threadIdx.x) * S + q]);
                norm[threadIdx.x] = nsum;
            }
            __syncthreads();
            float lmin = FLT_MAX;
            for (int i = threadIdx.x; i < rows * nOR; i += blockDim.x) {
                const int row = i / nOR, ior = i - row * nOR;
                const int tr = row / nOT, iot = row - tr * nOT;
                const long long e = job.off + ((long long)tr * nOR + ior) * nOT + iot;
                float csum = 0.f;
                for (int q = 0; q < S; ++q) csum += __ldcg(&qu.part[e * S + q]);
                const float v = norm[ior] - 2.f * csum;
                d[e] = v;
                ejob[e] = (int)jid;
                ecode[e] = ((unsigned)tlist[tr] * nOR + ior) * nOT + iot;
                lmin = fminf(lmin, v);
            }
            if (lmin < FLT_MAX) atomicMin(&smin, f2ord(lmin));
            __syncthreads();
            if (threadIdx.x == 0 && smin != 0xFFFFFFFFu) atomicMin(&ps[p].min_fine, smin);
        }
        __syncthreads();  // shared state of this item is done before the next item
    }
}

// One slice pixel's trilinear (3D) or bilinear (2D) insertion: value val,
// weight w, pixel (px, py), rotation Ai.
__device__ __forceinline__ void bp_insert(const float *Ai, int px, int py, float2 val, float w, const VolGeom &g,
                                          float4 *sv) {
    float xp = fmaf(Ai[0], (float)px, Ai[1] * (float)py);
    float yp = fmaf(Ai[3], (float)px, Ai[4] * (float)py);
    if (g.dim == 2) {
        // BackProjector::backrotate2D (src/backprojector.cpp:471-660):
        // bilinear insertion into the 2D data / weight planes
        if (xp < 0.f) {
            xp = -xp;
            yp = -yp;
            val.y = -val.y;
        }
        const float fx0 = floorf(xp), fy0 = floorf(yp);
        const float fx = xp - fx0, fy = yp - fy0;
        const int x0 = (int)fx0, y0 = (int)fy0 - g.yinit;
        if (x0 < 0 || x0 + 1 >= g.xdim || y0 < 0 || y0 + 1 >= g.ydim) return;
        const float mfx = 1.f - fx, mfy = 1.f - fy;
        const float d4[4] = {mfy * mfx, mfy * fx, fy * mfx, fy * fx};
        const size_t base = (size_t)y0 * g.xdim + x0;
        const size_t off4[4] = {0, 1, (size_t)g.xdim, (size_t)g.xdim + 1};
#pragma unroll
        for (int c = 0; c < 4; ++c)
            atomicAdd(&sv[base + off4[c]], make_float4(d4[c] * val.x, d4[c] * val.y, d4[c] * w, 0.f));
        return;
    }
    float zp = fmaf(Ai[6], (float)px, Ai[7] * (float)py);
    if (xp < 0.f) {
        xp = -xp;
        yp = -yp;
        zp = -zp;
        val.y = -val.y;
    }
    const float fx0 = floorf(xp), fy0 = floorf(yp), fz0 = floorf(zp);
    const float fx = xp - fx0, fy = yp - fy0, fz = zp - fz0;
    const int x0 = (int)fx0, y0 = (int)fy0 - g.yinit, z0 = (int)fz0 - g.zinit;
    if (x0 < 0 || x0 + 1 >= g.xdim || y0 < 0 || y0 + 1 >= g.ydim || z0 < 0 || z0 + 1 >= g.zdim) return;
    const float mfx = 1.f - fx, mfy = 1.f - fy, mfz = 1.f - fz;
    const float dd[8] = {mfz * mfy * mfx, mfz * mfy * fx, mfz * fy * mfx, mfz * fy * fx,
                         fz * mfy * mfx,  fz * mfy * fx,  fz * fy * mfx,  fz * fy * fx};
    const size_t sy = (size_t)g.xdim, sz = (size_t)g.xdim * g.ydim;
    const size_t base = (size_t)z0 * sz + (size_t)y0 * sy + x0;
    const size_t off[8] = {0, 1, sy, sy + 1, sz, sz + 1, sz + sy, sz + sy + 1};
#pragma unroll
    for (int c = 0; c < 8; ++c)
        atomicAdd(&sv[base + off[c]], make_float4(dd[c] * val.x, dd[c] * val.y, dd[c] * w, 0.f));
}

// ---------------------------------------------------------------------------
// storeWeightedSums for one job (particle p, coarse orientation r): for each
// oversampled orientation, the significant fine weights (w >= thr_fine,
// normalised by the sum) give W = sum w~ and the weighted phase sum
// Phi_k = sum w~ E_(t,iot),k, from which
//   sigma2 shell sums:  sum w~ |C P - X E|^2 (difference first, as the
//                       reference forms it per translation)
//   backprojection:     img += C Minv Xn Phi,  weight += W C^2 Minv
// (the per-translation sums of :8562-8780 rewritten with Phi).
// Blocks cover (job, chunk of kWsumPix x kWsumPer fine pixels), a thread per pixel at a time
// for all oversampled orientations, so each phase value is loaded once.
// ---------------------------------------------------------------------------
constexpr int kWsumPix = 128;
constexpr int kWsumPer = 4;
constexpr int kMaxOR = 8;

__global__ void __launch_bounds__(kWsumPix) k_wsum(WsumArgs a) {
    extern __shared__ double wsm[];
    double *shell = wsm;                                            // [nshell]
    float *wt = reinterpret_cast<float *>(shell + a.nshell);        // [rows][kMaxOR]
    int *tlist = reinterpret_cast<int *>(wt + a.T * a.nOT * kMaxOR); // [T]
    int *rlist = tlist + a.T;                                       // [rows] rows with a significant weight
    __shared__ double red[6];  // sumw, sigma2_offset, XA, AA, 2D class offset sums x / y
    __shared__ int wcount[kWsumPix / 32], nnz;
    __shared__ float Aj[kMaxOR][9];  // direct insertion: the job's slice rotations
    const FineJob job = a.jobs[blockIdx.x];
    const int p = job.p, r = job.r, n_t = job.n_t;
    const int nOR = a.nOR, nOT = a.nOT;
    const int rows = n_t * nOT;
    const bool first = blockIdx.y == 0;  // the per-job scalars are added once
    const float thr = a.ps[p].thr_fine;
    const double inv_sum = 1. / a.ps[p].sum_fine;
    const double *pd = a.pdat + (size_t)p * 8;
    const int ic = r / (a.ndir * a.npsi), idir = (r / a.npsi) % a.ndir;
    const float scale = a.do_scale ? fmaxf((float)pd[6], 0.001f) : 1.f;
    if (threadIdx.x == 0) {
        const unsigned int *mk = a.mask + ((size_t)p * a.R + r) * a.W;
        int m = 0;
        for (int w = 0; w < a.W; ++w) {
            unsigned int bits = mk[w];
            while (bits) {
                const int b = __ffs(bits) - 1;
                bits &= bits - 1;
                tlist[m++] = w * 32 + b;
            }
        }
    }
    if (threadIdx.x < 6) red[threadIdx.x] = 0.;
    if (threadIdx.x == 0) nnz = 0;
    if (a.bp_direct && threadIdx.x < nOR * 9)
        Aj[threadIdx.x / 9][threadIdx.x % 9] = a.eul_f[((size_t)r * nOR + threadIdx.x / 9) * 9 + threadIdx.x % 9];
    for (int i = threadIdx.x; i < a.nshell; i += blockDim.x) shell[i] = 0.;
    __syncthreads();
    // 2D classification: the offset prior is the class's (:8449-8456)
    const double prx = a.class_prior ? a.class_prior[2 * ic] : pd[2];
    const double pry = a.class_prior ? a.class_prior[2 * ic + 1] : pd[3];
    // normalised significant weights per (row, ior); FP64 scalar sums
    double l_sumw = 0., l_off = 0., l_px = 0., l_py = 0.;
    for (int i = threadIdx.x; i < rows * kMaxOR; i += blockDim.x) {
        const int row = i / kMaxOR, ior = i - row * kMaxOR;
        float wn = 0.f;
        if (ior < nOR) {
            const int tr = row / nOT, iot = row - tr * nOT;
            const long long e = job.off + ((long long)tr * nOR + ior) * nOT + iot;
            const float w = a.w[e];
            if (w > 0.f && w >= thr) {
                const double wd = (double)w * inv_sum;
                wn = (float)wd;
                l_sumw += wd;
                const int tf = tlist[tr] * nOT + iot;
                const double dx = prx - pd[0] - a.otx[tf];
                const double dy = pry - pd[1] - a.oty[tf];
                l_off += wd * a.pixel * a.pixel * dx * dx;
                l_off += wd * a.pixel * a.pixel * dy * dy;
                // class offset prior sums (:8668-8672)
                l_px += wd * a.pixel * (pd[0] + a.otx[tf]);
                l_py += wd * a.pixel * (pd[1] + a.oty[tf]);
            }
        }
        wt[i] = wn;
    }
    if (first) {
        l_sumw = warp_sum(l_sumw);
        l_off = warp_sum(l_off);
        l_px = warp_sum(l_px);
        l_py = warp_sum(l_py);
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&red[0], l_sumw);
            atomicAdd(&red[1], l_off);
            atomicAdd(&red[4], l_px);
            atomicAdd(&red[5], l_py);
        }
    }
    __syncthreads();
    // the rows (t, iot) with a significant weight for some orientation, in
    // row order (the sums below skip rows whose weights are all zero; adding
    // zero terms would not change them)
    {
        const int wp = threadIdx.x >> 5, ln = threadIdx.x & 31;
        for (int base = 0; base < rows; base += blockDim.x) {
            const int row = base + threadIdx.x;
            bool f = false;
            if (row < rows)
                for (int i = 0; i < nOR; ++i) f = f || wt[row * kMaxOR + i] != 0.f;
            const unsigned int bal = __ballot_sync(0xffffffffu, f);
            if (ln == 0) wcount[wp] = __popc(bal);
            __syncthreads();
            int off = nnz;
            for (int w2 = 0; w2 < wp; ++w2) off += wcount[w2];
            if (f) rlist[off + __popc(bal & ((1u << ln) - 1u))] = row;
            __syncthreads();
            if (threadIdx.x == 0)
                for (int w2 = 0; w2 < (int)(blockDim.x >> 5); ++w2) nnz += wcount[w2];
            __syncthreads();
        }
    }
    const int nrz = nnz;
    double l_xa = 0., l_aa = 0.;
    // kWsumPer pixels per thread: the job's weights, compaction and sums
    // above are made once per kWsumPer x kWsumPix pixels
    for (int sub = 0; sub < kWsumPer; ++sub) {
    const int k = (blockIdx.y * kWsumPer + sub) * kWsumPix + threadIdx.x;
    if (k < a.nf) {
        const float2 x = a.Xf[(size_t)p * a.nf + k], xn = a.Xnf[(size_t)p * a.nf + k];
        const float cs = a.Cf[(size_t)p * a.nf + k] * scale;
        const size_t rf0 = (size_t)r * nOR;
        float2 pv[kMaxOR], phi[kMaxOR];
        float s2[kMaxOR], W[kMaxOR];
#pragma unroll
        for (int ior = 0; ior < kMaxOR; ++ior) {
            pv[ior] = make_float2(0.f, 0.f);
            if (ior < nOR) pv[ior] = a.projf[(rf0 + ior) * a.ldpf + k];
            phi[ior] = make_float2(0.f, 0.f);
            s2[ior] = 0.f;
            W[ior] = 0.f;
        }
        for (int q = 0; q < nrz; ++q) {
            const int row = rlist[q];
            const int tr = row / nOT, iot = row - tr * nOT;
            const float2 e = a.phase_f[((size_t)tlist[tr] * nOT + iot) * a.nf + k];
            const float xr = x.x * e.x - x.y * e.y, xi = x.x * e.y + x.y * e.x;
            const float *wr = wt + row * kMaxOR;
#pragma unroll
            for (int ior = 0; ior < kMaxOR; ++ior) {
                const float wv = wr[ior];
                const float dr = fmaf(cs, pv[ior].x, -xr), di = fmaf(cs, pv[ior].y, -xi);
                s2[ior] = fmaf(wv, dr * dr + di * di, s2[ior]);
                phi[ior].x = fmaf(wv, e.x, phi[ior].x);
                phi[ior].y = fmaf(wv, e.y, phi[ior].y);
                W[ior] += wv;
            }
        }
        const int sh = a.pf[k].shell;
        const bool scale_shell = sh >= 0 && a.do_scale && a.dvp_mask[(size_t)ic * a.nshell + sh];
        const float minv = a.minv_store[k];
        const float f = cs * minv;
        // the pixel's sums over its kMaxOR orientations in FP32, FP64 from
        // there on (FP64 runs at a small fraction of the FP32 rate here)
        float s2tot = 0.f, xa = 0.f, aa = 0.f;
#pragma unroll
        for (int ior = 0; ior < kMaxOR; ++ior) {
            if (!(W[ior] > 0.f)) continue;
            const size_t rf = rf0 + ior;
            const float2 zx = make_float2(x.x * phi[ior].x - x.y * phi[ior].y, x.x * phi[ior].y + x.y * phi[ior].x);
            const float2 zn =
                make_float2(xn.x * phi[ior].x - xn.y * phi[ior].y, xn.x * phi[ior].y + xn.y * phi[ior].x);
            s2tot += s2[ior];
            if (scale_shell) {
                xa = fmaf(cs, pv[ior].x * zx.x + pv[ior].y * zx.y, xa);
                aa = fmaf(W[ior] * cs * cs, pv[ior].x * pv[ior].x + pv[ior].y * pv[ior].y, aa);
            }
            const float wgt = W[ior] * cs * cs * minv;
            if (a.bp_direct) {
                // the backprojection's pixel tests (k_backproject), then the
                // trilinear insertion of this slice pixel
                if (!(wgt > 0.f)) continue;
                const int px = a.pf[k].x, py = a.pf[k].y;
                const int rr = (int)lrintf((float)a.bg.r_max * a.bg.pad);
                if (a.bg.pad * a.bg.pad * (px * px + py * py) > rr * rr) continue;
                const int cb = a.circ ? a.circ[k] : -1;
                if (cb >= 0 && !((a.cmask[rf] >> cb) & 1ull)) continue;
                bp_insert(Aj[ior], px, py, make_float2(f * zn.x, f * zn.y), wgt, a.bg, a.stage[ic]);
                continue;
            }
            if (wgt != 0.f || f != 0.f) {
                atomicAdd(&a.bpimg[rf * a.nf + k].x, f * zn.x);
                atomicAdd(&a.bpimg[rf * a.nf + k].y, f * zn.y);
                atomicAdd(&a.bpw[rf * a.nf + k], wgt);
            }
            if (first && threadIdx.x == 0) a.active[rf] = 1;
        }
        if (scale_shell) {
            l_xa += (double)xa;
            l_aa += (double)aa;
        }
        if (sh >= 0 && s2tot != 0.f) atomicAdd(&shell[sh], (double)s2tot);
    }
    }
    if (a.do_scale) {
        l_xa = warp_sum(l_xa);
        l_aa = warp_sum(l_aa);
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&red[2], l_xa);
            atomicAdd(&red[3], l_aa);
        }
    }
    __syncthreads();
    double *sp = a.shell + (size_t)p * a.nshell;
    for (int i = threadIdx.x; i < a.nshell; i += blockDim.x)
        if (shell[i] != 0.) atomicAdd(&sp[i], shell[i]);
    if (threadIdx.x == 0) {
        double *pa = a.pacc + (size_t)p * 8;
        if (first) {
            atomicAdd(&pa[0], red[0]);
            atomicAdd(&pa[1], red[1]);
            atomicAdd(&a.pdf_dir[(size_t)ic * a.ndir + idir], red[0]);
            atomicAdd(&a.pdf_cls[ic], red[0]);
            if (a.w_prior_off) {
                atomicAdd(&a.w_prior_off[2 * ic], red[4]);
                atomicAdd(&a.w_prior_off[2 * ic + 1], red[5]);
            }
        }
        if (a.do_scale) {
            atomicAdd(&pa[2], red[2]);
            atomicAdd(&pa[3], red[3]);
        }
    }
}

__global__ void k_compact_flags(const unsigned char *__restrict__ flags, int n, int *__restrict__ list,
                                int *__restrict__ count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && flags[i]) {
        const int pos = atomicAdd(count, 1);
        list[pos] = i;
    }
}

// Trilinear insertion of the accumulated 2D slices of the active fine
// orientations (backproject2Dto3D, src/backprojector.cpp:55-296) into the
// FP32 staging volume: one float4 (re, im, weight, 0) per voxel, one vector
// atomic per corner (8 per pixel instead of 24 FP64 atomics); k_bp_flush adds
// the staging volume into the FP64 data and weight volumes once it holds a
// set number of particles (a few batches), so the volumes accumulate in FP64
// and a staging sum holds a bounded number of particles.  Each block handles
// one slice at a time; the slice accumulators are cleared for the next batch.
// A thread takes kBpUnroll pixels per step and issues their loads first: the
// kernel waits on those loads (slices scattered over the accumulator array),
// not on the atomics, so loads in flight per thread set its speed.
constexpr int kBpThreads = 256, kBpUnroll = 4;

__global__ void __launch_bounds__(kBpThreads)
k_backproject(const int *__restrict__ list, const float *__restrict__ eul_f, int nOR,
              const int *__restrict__ cls_of_r, float2 *__restrict__ bpimg, float *__restrict__ bpw,
              const PixelRef *__restrict__ pf, int nf, const VolGeom g, float4 *const *__restrict__ stage,
              unsigned char *__restrict__ active, const int *__restrict__ count, const int *__restrict__ circ,
              const unsigned long long *__restrict__ cmask) {
    const int nlist = *count;
    __shared__ float Ai[9];
    const int rr = (int)lrintf((float)g.r_max * g.pad);   // ROUND(r_max * pad)
    const int max_r2 = rr * rr;
    for (int li = blockIdx.x; li < nlist; li += gridDim.x) {
        const int rf = list[li];
        __syncthreads();  // the previous slice's readers of Ai are done
        if (threadIdx.x < 9) Ai[threadIdx.x] = eul_f[(size_t)rf * 9 + threadIdx.x];
        __syncthreads();
        float4 *sv = stage[cls_of_r[rf / nOR]];
        const unsigned long long cm = circ ? cmask[rf] : 0ull;
        for (int k0 = threadIdx.x; k0 < nf; k0 += kBpThreads * kBpUnroll) {
            float wv[kBpUnroll];
            float2 vv[kBpUnroll];
            int2 xy[kBpUnroll];
            int cb[kBpUnroll];
#pragma unroll
            for (int u = 0; u < kBpUnroll; ++u) {
                const int k = k0 + u * kBpThreads;
                wv[u] = 0.f;
                if (k < nf) {
                    const size_t idx = (size_t)rf * nf + k;
                    wv[u] = bpw[idx];
                    vv[u] = bpimg[idx];
                    xy[u] = *reinterpret_cast<const int2 *>(&pf[k]);
                    cb[u] = circ ? circ[k] : -1;
                }
            }
#pragma unroll
            for (int u = 0; u < kBpUnroll; ++u) {
                const int k = k0 + u * kBpThreads;
                if (k < nf) {
                    const size_t idx = (size_t)rf * nf + k;
                    bpw[idx] = 0.f;
                    bpimg[idx] = make_float2(0.f, 0.f);
                }
            }
#pragma unroll
            for (int u = 0; u < kBpUnroll; ++u) {
                if (!(wv[u] > 0.f)) continue;
                if (g.pad * g.pad * (xy[u].x * xy[u].x + xy[u].y * xy[u].y) > max_r2) continue;
                // pixels on the r_max circle: inserted where the reference inserts them
                if (cb[u] >= 0 && !((cm >> cb[u]) & 1ull)) continue;
                bp_insert(Ai, xy[u].x, xy[u].y, vv[u], wv[u], g, sv);
            }
        }
        if (threadIdx.x == 0) active[rf] = 0;
    }
}

// Adds one batch's FP32 staging volume into the FP64 data and weight
// volumes and clears it.  Only voxels within r_max pad + 2 of the origin can
// hold insertions (pixels inside r_max, trilinear corners one voxel out); the
// others are not read, and voxels no slice touched are only read.
__global__ void k_bp_flush(float4 *__restrict__ stage, double2 *__restrict__ data, double *__restrict__ weight,
                           const VolGeom g) {
    const size_t nvox = (size_t)g.xdim * g.ydim * g.zdim;
    const int rlim = g.r_max * g.pad + 2;
    for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(v % g.xdim);
        const size_t yz = v / g.xdim;
        const int y = (int)(yz % g.ydim) + g.yinit, z = (int)(yz / g.ydim) + g.zinit;
        if (x * x + y * y + z * z > rlim * rlim) continue;
        const float4 s = stage[v];
        if (s.x != 0.f || s.y != 0.f || s.z != 0.f) {
            double2 dv = data[v];
            dv.x += (double)s.x;
            dv.y += (double)s.y;
            data[v] = dv;
            weight[v] += (double)s.z;
            stage[v] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}

// ---------------------------------------------------------------------------
// Dense fine pass (most coarse poses significant): the fine diff2 / weight
// array is [p][rf][tf] over all oversampled orientations rf = r*nOR + ior
// and translations tf = t*nOT + iot.
// ---------------------------------------------------------------------------

// Normalise the fine weights in place: W = w / sum where w >= the fine
// significant weight, else 0 (storeWeightedSums :8562-8566); row sums per
// oversampled orientation (into Wt [rf][ldwt] and Wp [p][RF]), FP64 scalar
// sums (sum of W, sigma2_offset) and the pdf_direction / pdf_class sums.
// One block per (coarse orientation r, particle p).
__global__ void k_fine_normalize(float *__restrict__ w, int R, int nOR, int nOT, int T,
                                 const ParticleState *__restrict__ ps, const double *__restrict__ pdat,
                                 const double *__restrict__ otx, const double *__restrict__ oty,
                                 double pixel, int ndir, int npsi, float *__restrict__ Wt, int ldwt,
                                 float *__restrict__ Wp, int ldwp, unsigned char *__restrict__ active,
                                 double *__restrict__ pacc, double *__restrict__ pdf_dir,
                                 double *__restrict__ pdf_cls, const double *__restrict__ class_prior,
                                 double *__restrict__ w_prior_off) {
    __shared__ double rs[8];
    __shared__ double red[4];
    const int r = blockIdx.x, p = blockIdx.y;
    const int TF = T * nOT, RF = R * nOR;
    const float thr = ps[p].thr_fine;
    const double inv = 1. / ps[p].sum_fine;
    const double *pd = pdat + (size_t)p * 8;
    float *base = w + ((size_t)p * RF + (size_t)r * nOR) * TF;
    if (threadIdx.x < 8) rs[threadIdx.x] = 0.;
    if (threadIdx.x < 4) red[threadIdx.x] = 0.;
    __syncthreads();
    const int icl = r / (ndir * npsi);
    // 2D classification: the offset prior is the class's (:8449-8456)
    const double prx = class_prior ? class_prior[2 * icl] : pd[2];
    const double pry = class_prior ? class_prior[2 * icl + 1] : pd[3];
    double loff = 0., lpx = 0., lpy = 0.;
    double lrow[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) lrow[i] = 0.;
    for (int e = threadIdx.x; e < nOR * TF; e += blockDim.x) {
        const int ior = e / TF, tf = e - ior * TF;
        const float v = base[e];
        float wn = 0.f;
        if (v > 0.f && v >= thr) {
            const double wd = (double)v * inv;
            wn = (float)wd;
            const double dx = prx - pd[0] - otx[tf];
            const double dy = pry - pd[1] - oty[tf];
            loff += wd * pixel * pixel * dx * dx;
            loff += wd * pixel * pixel * dy * dy;
            lpx += wd * pixel * (pd[0] + otx[tf]);
            lpy += wd * pixel * (pd[1] + oty[tf]);
#pragma unroll
            for (int i = 0; i < 8; ++i)
                if (i == ior) lrow[i] += wd;
        }
        base[e] = wn;
    }
    loff = warp_sum(loff);
    lpx = warp_sum(lpx);
    lpy = warp_sum(lpy);
#pragma unroll
    for (int i = 0; i < 8; ++i) lrow[i] = warp_sum(lrow[i]);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&red[1], loff);
        atomicAdd(&red[2], lpx);
        atomicAdd(&red[3], lpy);
        for (int i = 0; i < nOR && i < 8; ++i)
            if (lrow[i] != 0.) atomicAdd(&rs[i], lrow[i]);
    }
    __syncthreads();
    if (threadIdx.x < nOR) {
        const int rf = r * nOR + threadIdx.x;
        const float v = (float)rs[threadIdx.x];
        Wt[(size_t)rf * ldwt + p] = v;
        Wp[(size_t)p * ldwp + rf] = v;
        if (v > 0.f) active[rf] = 1;
    }
    if (threadIdx.x == 0) {
        double tot = 0.;
        for (int i = 0; i < nOR && i < 8; ++i) tot += rs[i];
        if (tot != 0.) {
            const int ic = r / (ndir * npsi), idir = (r / npsi) % ndir;
            atomicAdd(&pacc[(size_t)p * 8 + 0], tot);
            atomicAdd(&pdf_dir[(size_t)ic * ndir + idir], tot);
            atomicAdd(&pdf_cls[ic], tot);
        }
        if (red[1] != 0.) atomicAdd(&pacc[(size_t)p * 8 + 1], red[1]);
        if (w_prior_off && (red[2] != 0. || red[3] != 0.)) {
            atomicAdd(&w_prior_off[2 * icl], red[2]);
            atomicAdd(&w_prior_off[2 * icl + 1], red[3]);
        }
    }
}

// B operand of the BP-slice contraction, stored transposed for K-contiguous
// rows: Zt[2k+c][(p,tf)] = Re/Im(C_pk s Minv_k Xn_pk E_tf,k); and
// CM[k][p] = (C_pk s)^2 Minv_k for the BP-weight contraction.
__global__ void k_make_zt(const float *__restrict__ Cf, const float2 *__restrict__ Xnf,
                          const float *__restrict__ minv_s, const float2 *__restrict__ E,
                          const double *__restrict__ pdat, int do_scale, int n, int TF, int nf,
                          float *__restrict__ Zt, long long ldz, float *__restrict__ CM, int ldcm) {
    const int k = blockIdx.y;
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const float ms = minv_s[k];
    if (j < ldz) {
        float zr = 0.f, zi = 0.f;
        if (j < (long long)n * TF) {
            const int p = (int)(j / TF), tf = (int)(j - (long long)p * TF);
            const float s = do_scale ? fmaxf((float)pdat[(size_t)p * 8 + 6], 0.001f) : 1.f;
            const float f = Cf[(size_t)p * nf + k] * s * ms;
            const float2 x = Xnf[(size_t)p * nf + k], e = __ldg(E + (size_t)tf * nf + k);
            zr = f * (x.x * e.x - x.y * e.y);
            zi = f * (x.x * e.y + x.y * e.x);
        }
        Zt[(size_t)(2 * k) * ldz + j] = zr;
        Zt[(size_t)(2 * k + 1) * ldz + j] = zi;
    }
    if (blockIdx.x == 0)
        for (int p = threadIdx.x; p < ldcm; p += blockDim.x) {
            float v = 0.f;
            if (p < n) {
                const float s = do_scale ? fmaxf((float)pdat[(size_t)p * 8 + 6], 0.001f) : 1.f;
                const float c = Cf[(size_t)p * nf + k] * s;
                v = c * c * ms;
            }
            CM[(size_t)k * ldcm + p] = v;
        }
}

// sigma2 shell sums of the dense path, one block per particle:
//   sum_poses W |C P - X E|^2 = C^2 S - 2 C Re(conj(X) G) + (sum W) |X|^2
// per pixel, binned by resolution shell (plus the scale-correction sums).
__global__ void k_shell_dense(const float *__restrict__ S2P, const float2 *__restrict__ G,
                              const float2 *__restrict__ Xf, const float *__restrict__ Cf,
                              const PixelRef *__restrict__ pf, int nf, int nshell,
                              const double *__restrict__ pdat, int do_scale,
                              const unsigned char *__restrict__ dvp_mask, int K, int ic_single,
                              double *__restrict__ pacc, double *__restrict__ shell) {
    extern __shared__ double ssh[];
    __shared__ double red[2];
    const int p = blockIdx.x;
    for (int i = threadIdx.x; i < nshell; i += blockDim.x) ssh[i] = 0.;
    if (threadIdx.x < 2) red[threadIdx.x] = 0.;
    __syncthreads();
    const double wtot = pacc[(size_t)p * 8 + 0];
    const float s = do_scale ? fmaxf((float)pdat[(size_t)p * 8 + 6], 0.001f) : 1.f;
    double lxa = 0., laa = 0.;
    for (int k = threadIdx.x; k < nf; k += blockDim.x) {
        const int sh = pf[k].shell;
        if (sh < 0) continue;
        const float c = Cf[(size_t)p * nf + k] * s;
        const float2 x = Xf[(size_t)p * nf + k], g = G[(size_t)p * nf + k];
        const double sp = S2P[(size_t)p * nf + k];
        const double cross = (double)x.x * g.x + (double)x.y * g.y;
        const double v = (double)c * c * sp - 2.0 * c * cross + wtot * ((double)x.x * x.x + (double)x.y * x.y);
        atomicAdd(&ssh[sh], v);
        if (do_scale && K == 1 && dvp_mask[(size_t)ic_single * nshell + sh]) {
            lxa += (double)c * cross;
            laa += (double)c * c * sp;
        }
    }
    if (do_scale) {
        lxa = warp_sum(lxa);
        laa = warp_sum(laa);
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&red[0], lxa);
            atomicAdd(&red[1], laa);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nshell; i += blockDim.x)
        if (ssh[i] != 0.) shell[(size_t)p * nshell + i] += ssh[i];
    if (threadIdx.x == 0 && do_scale) {
        pacc[(size_t)p * 8 + 2] += red[0];
        pacc[(size_t)p * 8 + 3] += red[1];
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// launch wrappers
// ---------------------------------------------------------------------------
cudaError_t launch_prep(const float2 *X, const float *C, const double *pdat, int n, int full_npix,
                        const PixelRef *pc, int nc, const float *minv_c, int ldk_c,
                        const PixelRef *pf, int nf, int ldk_f, const float *minv_f, float *a_c, float2 *b_c,
                        float *a_f, float2 *b_f, float2 *Xf, float2 *Xnf, float *Cf,
                        const float2 *Xn, int do_scale, ParticleState *ps, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_prep<<<n, 512, 0, st>>>(X, C, Xn, pdat, full_npix, pc, nc, minv_c, ldk_c, pf, nf, ldk_f, minv_f, a_c,
                              b_c, a_f, b_f, Xf, Xnf, Cf, do_scale, ps);
    return cudaGetLastError();
}

cudaError_t launch_pdf_offset(const double *pdat, int n, const double *tx, const double *ty, int T,
                              double sigma2_offset, double pixel, float *pdf_off, double log_rt_orient,
                              ParticleState *ps, int KP, const double *class_prior, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const size_t smem = sizeof(double) * (size_t)KP * T;
    if (smem > 200 * 1024) return cudaErrorInvalidValue;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_pdf_offset, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    k_pdf_offset<<<n, 256, smem, st>>>(pdat, tx, ty, T, sigma2_offset, pixel, pdf_off, log_rt_orient, ps, KP,
                                       class_prior);
    return cudaGetLastError();
}

static size_t hist_smem() { return kHistBins * (sizeof(double) + sizeof(unsigned int)); }

cudaError_t launch_weights(float *vals, const long long *seg, int n, long long max_len, int coarse,
                           int T, const int *ejob, const unsigned int *ecode, const FineJob *jobs,
                           int nOR, int nOT, const float *pdf_orient, const float *pdf_off,
                           ParticleState *ps, HistBin *hist, cudaStream_t st, int add_sum, int KP, int rpc,
                           const unsigned int *segmask) {
    (void)hist;
    if (n <= 0 || max_len <= 0) return cudaSuccess;
    const long long nb = (max_len + kChunk - 1) / kChunk;
    if (nb > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    dim3 grid((unsigned)nb, n);
    k_weights<<<grid, kWThreads, 0, st>>>(vals, seg, coarse, T, ejob, ecode, jobs, nOR, nOT, pdf_orient,
                                          pdf_off, ps, add_sum, KP, rpc, segmask);
    return cudaGetLastError();
}

cudaError_t launch_hist_refine(const float *vals, const long long *seg, int n, long long max_len,
                               int level, ParticleState *ps, HistBin *hist, cudaStream_t st, int pass,
                               double fraction, const long long *seg_end, long long n_total) {
    if (n <= 0 || max_len <= 0) return cudaSuccess;
    const long long nb = (max_len + kChunk - 1) / kChunk;
    dim3 grid((unsigned)nb, n);
    k_hist_refine<<<grid, kWThreads, hist_smem(), st>>>(vals, seg, level, ps, hist, pass, fraction, seg_end,
                                                        n_total);
    return cudaGetLastError();
}

size_t select_fused_smem() { return kHistBins * (sizeof(double) + sizeof(unsigned int)) +
                                     kSelThreads * (sizeof(double) + sizeof(unsigned int)); }

cudaError_t launch_select_fused(const float *vals, const long long *seg, const long long *seg_end, int n,
                                long long n_total, int pass, double fraction, int coarse, ParticleState *ps,
                                cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_select_fused, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)select_fused_smem());
        if (e != cudaSuccess) return e;
        attr = true;
    }
    k_select_fused<<<n, kSelThreads, select_fused_smem(), st>>>(vals, seg, seg_end, n_total, pass, fraction, coarse,
                                                                 ps);
    return cudaGetLastError();
}

cudaError_t launch_select(int n, int level, double adaptive_fraction, int coarse, ParticleState *ps,
                          HistBin *hist, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_select<<<n, 256, 0, st>>>(level, adaptive_fraction, coarse, ps, hist);
    return cudaGetLastError();
}

cudaError_t launch_sig_masks(const float *w, int n, int R, int T, int W, const ParticleState *ps,
                             unsigned int *mask, int *cnt, cudaStream_t st) {
    const long long warps = (long long)n * R;
    if (warps <= 0) return cudaSuccess;
    const long long blocks = (warps * 32 + 255) / 256;
    k_sig_masks<<<(unsigned)blocks, 256, 0, st>>>(w, n, R, T, W, ps, mask, cnt);
    return cudaGetLastError();
}

cudaError_t launch_fine_jobs(const int *cnt, int n, int R, int per, long long *sums, FineJob *jobs, long long *seg,
                             unsigned char *need_r, cudaStream_t st) {
    const long long tot = (long long)n * R;
    if (tot <= 0) return cudaSuccess;
    const long long nb = fine_jobs_nblocks(tot);
    if (nb > 0x7fffffffLL) return cudaErrorInvalidValue;
    k_jobs_reduce<<<(unsigned)nb, kJobsThreads, 0, st>>>(cnt, tot, per, sums);
    k_jobs_scan_sums<<<1, kScanBlock, 0, st>>>(sums, (int)nb);
    k_jobs_emit<<<(unsigned)nb, kJobsThreads, 0, st>>>(cnt, n, R, per, sums, (int)nb, jobs, seg, need_r);
    return cudaGetLastError();
}

// After a pass: the significance mask words and counts of every job's row
// back to zero (the rows with a nonzero count are exactly the jobs), so the
// next pass starts from clear arrays without a full memset.
__global__ void k_clear_job_rows(const FineJob *__restrict__ jobs, const long long *__restrict__ njobs, int R,
                                 int W, unsigned int *__restrict__ mask, int *__restrict__ cnt) {
    const long long nj = *njobs;
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < nj;
         j += (long long)gridDim.x * blockDim.x) {
        const FineJob jb = jobs[j];
        const size_t row = (size_t)jb.p * R + jb.r;
        cnt[row] = 0;
        for (int k = 0; k < W; ++k) mask[row * W + k] = 0u;
    }
}

cudaError_t launch_clear_job_rows(const FineJob *jobs, const long long *njobs_dev, long long njobs_max, int R, int W,
                                  unsigned int *mask, int *cnt, cudaStream_t st) {
    if (njobs_max <= 0) return cudaSuccess;
    const int grid = (int)std::min<long long>((njobs_max + 255) / 256, 4096);
    k_clear_job_rows<<<grid, 256, 0, st>>>(jobs, njobs_dev, R, W, mask, cnt);
    return cudaGetLastError();
}

long long fine_jobs_nblocks(long long tot) {
    const long long per_block = (long long)kJobsThreads * kJobsPer;
    return (tot + per_block - 1) / per_block;
}

int fine_diff2_nsplit(int nf) { return (nf + kFineSplit - 1) / kFineSplit; }

cudaError_t launch_fine_diff2(const FineJob *jobs, const long long *njobs_dev, long long njobs_max, int nsplit,
                              unsigned long long *head, int *arrive, float *part, float *npart,
                              const unsigned int *mask, int R, int T, int W, int nOR, int nOT, const float2 *projf,
                              int ldpf, const float2 *b_f, const float *a_f, int nf, const float2 *phase_f, float *d,
                              int *ejob, unsigned int *ecode, ParticleState *ps, cudaStream_t st) {
    if (njobs_max <= 0) return cudaSuccess;
    if (nOR > 8 || nsplit != fine_diff2_nsplit(nf)) return cudaErrorInvalidValue;
    const size_t smem = sizeof(float2) * 8 * kFineChunk + sizeof(float) * T * nOT * nOR +
                        sizeof(int) * T + sizeof(float) * nOR + 16;
    static size_t attr = 0;
    static int slots = 0;
    if (smem > attr) {
        cudaError_t e = cudaFuncSetAttribute(k_fine_diff2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr = smem;
        slots = 0;
    }
    if (!slots) {
        // persistent grid: as many blocks as fit on the device at once
        int dev = 0, nsm = 0, per = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_fine_diff2, kFineThreads, smem);
        if (e != cudaSuccess) return e;
        slots = std::max(1, nsm * std::max(per, 1));
    }
    cudaError_t e = cudaMemsetAsync(head, 0, sizeof(unsigned long long), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(arrive, 0, sizeof(int) * njobs_max, st);
    if (e != cudaSuccess) return e;
    const long long items = njobs_max * nsplit;
    const int grid = (int)std::min<long long>(items, slots);
    const FineQueue qu{njobs_dev, nsplit, head, arrive, part, npart};
    k_fine_diff2<<<grid, kFineThreads, smem, st>>>(jobs, qu, mask, R, T, W, nOR, nOT, projf, ldpf, b_f, a_f, nf,
                                                   phase_f, d, ejob, ecode, ps);
    return cudaGetLastError();
}

cudaError_t launch_wsum(const WsumArgs &a, cudaStream_t st) {
    if (a.njobs <= 0) return cudaSuccess;
    if (a.nOR > kMaxOR) return cudaErrorInvalidValue;
    if (a.njobs > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    const size_t smem = sizeof(double) * a.nshell + sizeof(float) * (size_t)kMaxOR * a.T * a.nOT +
                        sizeof(int) * (a.T + (size_t)a.T * a.nOT) + 16;
    static size_t attr = 0;
    if (smem > attr) {
        cudaError_t e = cudaFuncSetAttribute(k_wsum, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr = smem;
    }
    dim3 grid((unsigned)a.njobs, (unsigned)((a.nf + kWsumPix * kWsumPer - 1) / (kWsumPix * kWsumPer)));
    k_wsum<<<grid, kWsumPix, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_compact_flags(const unsigned char *flags, int n, int *list, int *count,
                                 cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_compact_flags<<<(n + 255) / 256, 256, 0, st>>>(flags, n, list, count);
    return cudaGetLastError();
}

cudaError_t launch_bp_flush(float4 *stage, double2 *data, double *weight, const VolGeom &g, cudaStream_t st) {
    const size_t nvox = (size_t)g.xdim * g.ydim * g.zdim;
    if (nvox == 0) return cudaSuccess;
    int dev = 0, nsm = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const size_t blocks = std::min<size_t>((nvox + 255) / 256, (size_t)nsm * 16);
    k_bp_flush<<<(unsigned)blocks, 256, 0, st>>>(stage, data, weight, g);
    return cudaGetLastError();
}

cudaError_t launch_backproject(const int *list, const int *count, int max_list, const float *eul_f, int nOR,
                               const int *cls_of_r, float2 *bpimg, float *bpw, const PixelRef *pf, int nf,
                               const VolGeom &g, float4 *const *stage, unsigned char *active, cudaStream_t st,
                               const int *circ, const unsigned long long *mask) {
    if (max_list <= 0) return cudaSuccess;
    if ((circ == nullptr) != (mask == nullptr)) return cudaErrorInvalidValue;
    // slices are read from the device-side list; the grid covers the device
    // a few times over and loops over the slices present
    int dev = 0, nsm = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int grid = std::min(max_list, 8 * nsm);
    k_backproject<<<grid, kBpThreads, 0, st>>>(list, eul_f, nOR, cls_of_r, bpimg, bpw, pf, nf, g, stage, active,
                                                count, circ, mask);
    return cudaGetLastError();
}

// Per-particle metadata rows pdat[p] = {old_x, old_y, prior_x, prior_y,
// highres_Xi2, norm, scale, 0} from device-resident batch arrays.
__global__ void k_gather_pdat(const double *__restrict__ old_offset, const double *__restrict__ prior,
                              const double *__restrict__ xi2, const double *__restrict__ norm,
                              const double *__restrict__ scale, int n, double *__restrict__ pdat) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    double *o = pdat + (size_t)p * 8;
    o[0] = old_offset[2 * p];
    o[1] = old_offset[2 * p + 1];
    o[2] = prior[2 * p];
    o[3] = prior[2 * p + 1];
    o[4] = xi2[p];
    o[5] = norm[p];
    o[6] = scale[p];
    o[7] = 0.;
}

cudaError_t launch_gather_pdat(const double *old_offset, const double *prior, const double *xi2,
                               const double *norm, const double *scale, int n, double *pdat, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_gather_pdat<<<(n + 127) / 128, 128, 0, st>>>(old_offset, prior, xi2, norm, scale, n, pdat);
    return cudaGetLastError();
}

// Candidate-list segments: [p cap, p cap + min(count, cap)) per particle.
__global__ void k_cand_seg(const unsigned int *__restrict__ cnt, int n, int cap, long long *__restrict__ seg) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    seg[p] = (long long)p * cap;
    seg[n + p] = (long long)p * cap + (long long)min(cnt[p], (unsigned int)cap);
}

cudaError_t launch_cand_seg(const unsigned int *cnt, int n, int cap, long long *seg, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_cand_seg<<<(n + 127) / 128, 128, 0, st>>>(cnt, n, cap, seg);
    return cudaGetLastError();
}

cudaError_t launch_fine_normalize(float *w, int n, int R, int nOR, int nOT, int T, const ParticleState *ps,
                                  const double *pdat, const double *otx, const double *oty, double pixel,
                                  int ndir, int npsi, float *Wt, int ldwt, float *Wp, int ldwp, unsigned char *active,
                                  double *pacc, double *pdf_dir, double *pdf_cls, const double *class_prior,
                                  double *w_prior_off, cudaStream_t st) {
    if (n <= 0 || nOR > 8) return nOR > 8 ? cudaErrorInvalidValue : cudaSuccess;
    dim3 grid(R, n);
    k_fine_normalize<<<grid, 256, 0, st>>>(w, R, nOR, nOT, T, ps, pdat, otx, oty, pixel, ndir, npsi, Wt, ldwt,
                                           Wp, ldwp, active, pacc, pdf_dir, pdf_cls, class_prior, w_prior_off);
    return cudaGetLastError();
}

cudaError_t launch_make_zt(const float *Cf, const float2 *Xnf, const float *minv_s, const float2 *E,
                           const double *pdat, int do_scale, int n, int TF, int nf, float *Zt, long long ldz,
                           float *CM, int ldcm, cudaStream_t st) {
    if (n <= 0 || nf <= 0) return cudaSuccess;
    dim3 grid((unsigned)((ldz + 255) / 256), nf);
    k_make_zt<<<grid, 256, 0, st>>>(Cf, Xnf, minv_s, E, pdat, do_scale, n, TF, nf, Zt, ldz, CM, ldcm);
    return cudaGetLastError();
}

cudaError_t launch_shell_dense(int n, const float *S2P, const float2 *G, const float2 *Xf, const float *Cf,
                               const PixelRef *pf, int nf, int nshell, const double *pdat, int do_scale,
                               const unsigned char *dvp_mask, int K, double *pacc, double *shell,
                               cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_shell_dense<<<n, 256, sizeof(double) * nshell, st>>>(S2P, G, Xf, Cf, pf, nf, nshell, pdat, do_scale,
                                                           dvp_mask, K, 0, pacc, shell);
    return cudaGetLastError();
}


cudaError_t launch_weights_cand(const float *vals, int n, int R, int T, const float *pdf_orient, float pdf_orient_min,
                                const float *pdf_off, double fraction, ParticleState *ps, unsigned int *cand_idx,
                                float *cand_w, unsigned int *cand_cnt, int cap, float *dense_out,
                                const unsigned int *rowmin, int KP, int rpc, const unsigned int *segmask,
                                int cand_buf, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    // orientations per block: up to kWRowsPerBlock, fewer when the prior rows
    // of the classes a block touches ((rpb - 1) / rpc + 2 of them) would not
    // fit next to the 17 KB static candidate buffer
    const int max_cls = (int)((30 * 1024) / (sizeof(float) * (size_t)std::max(T, 1)));
    if (KP > 1 && max_cls < 2) return cudaErrorInvalidValue;
    const int rpb = KP > 1 ? std::max(1, std::min(kWRowsPerBlock, (max_cls - 1) * std::max(rpc, 1))) : kWRowsPerBlock;
    const int ncls = KP > 1 ? std::min(KP, (rpb - 1) / std::max(rpc, 1) + 2) : 1;
    const size_t smem = (size_t)ncls * T * sizeof(float);
    dim3 grid((unsigned)((R + rpb - 1) / rpb), n);
    k_weights_cand<<<grid, kWThreads, smem, st>>>(vals, R, T, pdf_orient, pdf_orient_min, pdf_off, fraction, ps,
                                                  cand_idx, cand_w, cand_cnt, cap, dense_out, rowmin, KP, rpc,
                                                  segmask, (cand_buf > 0 && cand_buf < kCandBuf) ? cand_buf : kCandBuf, rpb);
    return cudaGetLastError();
}

cudaError_t launch_cand_masks(const unsigned int *cand_idx, const float *cand_w, const unsigned int *cand_cnt,
                              int cap, int n, int R, int T, int W, const ParticleState *ps, unsigned int *mask,
                              int *cnt, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    dim3 grid(64, n);
    k_cand_masks<<<grid, 256, 0, st>>>(cand_idx, cand_w, cand_cnt, cap, R, T, W, ps, mask, cnt);
    return cudaGetLastError();
}

}  // namespace gbr
