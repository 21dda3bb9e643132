// Pose-proposal network: a small convolutional classifier of the viewing
// direction, trained and run by the kernels below (no library calls).
//
// Input features of a particle: its whitened coarse power |X_j|^2 / sigma2_j
// over the active coarse pixels (the pixels the E-step scores), averaged in
// polar bins (ring = the pixel's shell 1..H, angle = atan2(y, x) modulo pi in
// W bins) and mapped to log(1 + mean) - log 2 (0 for pure noise, 0 in empty
// bins).  Power removes the translation; an in-plane rotation becomes a
// circular shift along the angle axis.
//
// Layers ([B][C][H][W] row-major, angle fastest):
//   conv1  1 -> C1, 3 x 5 kernel (zero padding along rings, circular along
//          angles), bias, ReLU
//   conv2  C1 -> C2, same, ReLU
//   pool   mean over angles  -> h [B][C2*H]   (invariant to in-plane rotation)
//   linear h W3 + b3         -> logits [B][ND] (one per HEALPix direction)
//   softmax cross entropy against a target distribution (one-hot labels of
//   the synthetic training views, or E-step posteriors)
// Parameters in one array: W1 [C1][1][3][5], b1 [C1], W2 [C2][C1][3][5],
// b2 [C2], W3 [C2*H][ND], b3 [ND].
//
// Training views are projections of the current reference taken from the
// coarse projection table (one row per coarse orientation, so the direction
// label is exact), multiplied by the CTF of a particle drawn from a pool and
// given complex Gaussian noise of the model's sigma2 per pixel.  Random
// numbers: SplitMix64 (Steele, Lea, Flood 2014) of (seed, step, sample,
// pixel), Box-Muller for the normals.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "gbr_internal.h"

namespace gbr {
namespace {

constexpr int KH = 3, KW = 5;
constexpr float kLn2 = 0.6931471805599453f;

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// uniform in (0, 1]
__device__ __forceinline__ float unit(uint64_t h) { return ((float)(h >> 40) + 1.f) * (1.f / 16777216.f); }

// Training views: whitened power of CTF * P_r + noise at the active pixels.
__global__ void k_pn_gen(const float *__restrict__ proj, int lda, const PixelRef *__restrict__ pix, int npix,
                         const float *__restrict__ minv, const float *__restrict__ ctf_pool, int full_npix,
                         int n_pool, long long R, int NP, int ND, uint64_t seed, float *__restrict__ v,
                         int *__restrict__ label) {
    const int b = blockIdx.x;
    __shared__ long long s_r;
    __shared__ int s_k;
    if (threadIdx.x == 0) {
        const uint64_t h = mix64(seed ^ mix64((uint64_t)b * 0x100000001B3ull));
        s_r = (long long)(h % (uint64_t)R);
        s_k = (int)(mix64(h) % (uint64_t)n_pool);
        label[b] = (int)((s_r / NP) % ND);
    }
    __syncthreads();
    const float *row = proj + (size_t)s_r * lda;
    const float *ctf = ctf_pool + (size_t)s_k * full_npix;
    for (int j = threadIdx.x; j < npix; j += blockDim.x) {
        const float c = ctf[pix[j].full];
        const float s2 = 0.5f / minv[j];  // minv = 1 / (2 sigma2)
        const uint64_t h = mix64(seed ^ mix64(((uint64_t)b << 32) ^ (uint64_t)j ^ 0xA5A5A5A5ull));
        const float u1 = unit(h), u2 = unit(mix64(h));
        const float rad = sqrtf(-2.f * logf(u1) * 0.5f * s2);
        float sn, cs;
        sincospif(2.f * u2, &sn, &cs);
        const float xr = c * row[2 * j] + rad * cs, xi = c * row[2 * j + 1] + rad * sn;
        v[(size_t)b * npix + j] = (xr * xr + xi * xi) / s2;
    }
}

// Whitened power of prepared particle images (fimg [B][full_npix] complex).
__global__ void k_pn_power(const float2 *__restrict__ fimg, int full_npix, const PixelRef *__restrict__ pix,
                           int npix, const float *__restrict__ minv, int B, float *__restrict__ v) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)B * npix) return;
    const int b = (int)(i / npix), j = (int)(i % npix);
    const float2 x = fimg[(size_t)b * full_npix + pix[j].full];
    v[i] = (x.x * x.x + x.y * x.y) * 2.f * minv[j];
}

// Polar bins: one block per sample, shared-memory sums.
__global__ void k_pn_bin(const float *__restrict__ v, int npix, const int *__restrict__ bin,
                         const float *__restrict__ inv_cnt, int nbins, float *__restrict__ feat) {
    extern __shared__ float acc[];
    const int b = blockIdx.x;
    for (int i = threadIdx.x; i < nbins; i += blockDim.x) acc[i] = 0.f;
    __syncthreads();
    for (int j = threadIdx.x; j < npix; j += blockDim.x) {
        const int k = bin[j];
        if (k >= 0) atomicAdd(&acc[k], v[(size_t)b * npix + j]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nbins; i += blockDim.x)
        feat[(size_t)b * nbins + i] = inv_cnt[i] > 0.f ? log1pf(acc[i] * inv_cnt[i]) - kLn2 : 0.f;
}

// out[b][co][y][x] = relu(bias[co] + sum W[co][ci][ky][kx] in[b][ci][y+ky-1][(x+kx-2) mod W])
// One thread per output position (b, y, x) computes every output channel:
// each input value is loaded once for all Co channels, the weights and
// biases sit in shared memory (read as broadcasts).  Per channel the sum
// runs over ci, then ky, then kx, as a one-output-per-thread form would.
constexpr int kPnMaxCo = 32;

__global__ void __launch_bounds__(256)
k_pn_conv_fwd(const float *__restrict__ in, int Ci, const float *__restrict__ w, const float *__restrict__ bias,
              int Co, int H, int W, int B, float *__restrict__ out) {
    extern __shared__ float wsh[];  // [Co][Ci][KH*KW], then bias[Co]
    const int nw = Co * Ci * KH * KW;
    for (int j = threadIdx.x; j < nw + Co; j += blockDim.x) wsh[j] = j < nw ? w[j] : bias[j - nw];
    __syncthreads();
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)B * H * W) return;
    const int x = (int)(i % W), y = (int)((i / W) % H), b = (int)(i / ((long long)W * H));
    float acc[kPnMaxCo];
#pragma unroll
    for (int co = 0; co < kPnMaxCo; ++co) acc[co] = co < Co ? wsh[nw + co] : 0.f;
    for (int ci = 0; ci < Ci; ++ci) {
        const float *src = in + ((size_t)b * Ci + ci) * H * W;
        float v[KH * KW];
        bool ok[KH];
#pragma unroll
        for (int ky = 0; ky < KH; ++ky) {
            const int yy = y + ky - 1;
            ok[ky] = yy >= 0 && yy < H;
#pragma unroll
            for (int kx = 0; kx < KW; ++kx) {
                int xx = x + kx - 2;
                xx += (xx < 0) ? W : 0;
                xx -= (xx >= W) ? W : 0;
                v[ky * KW + kx] = ok[ky] ? src[yy * W + xx] : 0.f;
            }
        }
#pragma unroll
        for (int co = 0; co < kPnMaxCo; ++co) {
            if (co >= Co) break;
            const float *wk = wsh + ((size_t)co * Ci + ci) * KH * KW;
            float s = acc[co];
#pragma unroll
            for (int ky = 0; ky < KH; ++ky) {
                if (!ok[ky]) continue;
#pragma unroll
                for (int kx = 0; kx < KW; ++kx) s += wk[ky * KW + kx] * v[ky * KW + kx];
            }
            acc[co] = s;
        }
    }
#pragma unroll
    for (int co = 0; co < kPnMaxCo; ++co)
        if (co < Co) {
            const float s = acc[co];
            out[(((size_t)b * Co + co) * H + y) * W + x] = s > 0.f ? s : 0.f;
        }
}

// h[b][c*H + y] = mean over x of a[b][c][y][x]
__global__ void k_pn_pool(const float *__restrict__ a, int C, int H, int W, int B, float *__restrict__ h) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)B * C * H) return;
    const float *src = a + (size_t)i * W;
    float s = 0.f;
    for (int x = 0; x < W; ++x) s += src[x];
    h[i] = s / (float)W;
}

// logits[b][n] = b3[n] + sum_f h[b][f] W3[f][n]
__global__ void k_pn_linear(const float *__restrict__ h, int F, const float *__restrict__ w,
                            const float *__restrict__ bias, int N, int B, float *__restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)B * N) return;
    const int n = (int)(i % N), b = (int)(i / N);
    const float *hb = h + (size_t)b * F;
    float s = bias[n];
    for (int f = 0; f < F; ++f) s += hb[f] * w[(size_t)f * N + n];
    out[i] = s;
}

__device__ float block_reduce(float v, float *sh, bool is_max) {
    for (int o = 16; o > 0; o >>= 1) {
        const float u = __shfl_xor_sync(0xffffffffu, v, o);
        v = is_max ? fmaxf(v, u) : v + u;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    float r = is_max ? -3.4e38f : 0.f;
    for (int k = 0; k < nw; ++k) r = is_max ? fmaxf(r, sh[k]) : r + sh[k];
    return r;
}

// Softmax cross entropy, one block per sample.  Target: one-hot `label` if
// given, else the distribution `target` [B][N].  dl = (softmax - t) / B.
__global__ void k_pn_xent(const float *__restrict__ logits, int N, const int *__restrict__ label,
                          const float *__restrict__ target, int B, float *__restrict__ dl, float *__restrict__ loss) {
    __shared__ float sh[32];
    const int b = blockIdx.x;
    const float *l = logits + (size_t)b * N;
    float m = -3.4e38f;
    for (int n = threadIdx.x; n < N; n += blockDim.x) m = fmaxf(m, l[n]);
    m = block_reduce(m, sh, true);
    float se = 0.f;
    for (int n = threadIdx.x; n < N; n += blockDim.x) se += expf(l[n] - m);
    se = block_reduce(se, sh, false);
    const float lse = m + logf(se);
    float ls = 0.f;
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        const float t = label ? (n == label[b] ? 1.f : 0.f) : target[(size_t)b * N + n];
        const float p = expf(l[n] - lse);
        dl[(size_t)b * N + n] = (p - t) / (float)B;
        ls += t * (lse - l[n]);
    }
    ls = block_reduce(ls, sh, false);
    if (threadIdx.x == 0) loss[b] = ls;
}

// dW3[f][n] = sum_b h[b][f] dl[b][n]; row f = F holds db3[n] = sum_b dl[b][n]
__global__ void k_pn_linear_bwd_w(const float *__restrict__ h, const float *__restrict__ dl, int F, int N, int B,
                                  float *__restrict__ dw, float *__restrict__ db) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)(F + 1) * N) return;
    const int n = (int)(i % N), f = (int)(i / N);
    float s = 0.f;
    if (f < F) {
        for (int b = 0; b < B; ++b) s += h[(size_t)b * F + f] * dl[(size_t)b * N + n];
        dw[(size_t)f * N + n] = s;
    } else {
        for (int b = 0; b < B; ++b) s += dl[(size_t)b * N + n];
        db[n] = s;
    }
}

// dh[b][f] = sum_n dl[b][n] W3[f][n]; through the mean pool and the ReLU of
// a2: d2[b][c][y][x] = dh[b][c*H + y] / W * (a2 > 0)
__global__ void k_pn_linear_bwd_x(const float *__restrict__ dl, const float *__restrict__ w, int F, int N, int B,
                                  const float *__restrict__ a2, int W, float *__restrict__ d2) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)B * F) return;
    const int f = (int)(i % F), b = (int)(i / F);
    const float *dlb = dl + (size_t)b * N;
    const float *wf = w + (size_t)f * N;
    float s = 0.f;
    for (int n = 0; n < N; ++n) s += dlb[n] * wf[n];
    s /= (float)W;
    const float *ab = a2 + (size_t)i * W;
    float *db = d2 + (size_t)i * W;
    for (int x = 0; x < W; ++x) db[x] = ab[x] > 0.f ? s : 0.f;
}

// Weight and bias gradients of a convolution, in two deterministic steps:
// block k of k_pn_conv_bwd_w_part accumulates, for particles k, k + grid, ...,
// every gradient entry (co, ci, ky, kx), then the biases (co), over row
// tiles staged in shared memory (inputs with their halo rows, output
// gradients); thread t owns entries t, t + kBwThreads, ...  k_pn_sum_parts
// adds the blocks' partial sums in block order.
constexpr int kBwThreads = 1024, kBwPer = 16;  // up to 16,384 entries
constexpr int kBwParts = 256;                 // partial-sum blocks at most

__global__ void __launch_bounds__(kBwThreads)
k_pn_conv_bwd_w_part(const float *__restrict__ in, int Ci, const float *__restrict__ d, int Co, int H, int W, int B,
                     int rows, float *__restrict__ part) {
    extern __shared__ float bsm[];
    float *sin = bsm;                           // [Ci][rows + 2][W]
    float *sd = bsm + (size_t)Ci * (rows + 2) * W;  // [Co][rows][W]
    const int nw = Co * Ci * KH * KW, nent = nw + Co;
    float acc[kBwPer];
#pragma unroll
    for (int j = 0; j < kBwPer; ++j) acc[j] = 0.f;
    for (int b = blockIdx.x; b < B; b += gridDim.x) {
        for (int y0 = 0; y0 < H; y0 += rows) {
            const int ry = min(rows, H - y0);
            __syncthreads();  // the previous tile's readers are done
            for (int i = threadIdx.x; i < Ci * (ry + 2) * W; i += blockDim.x) {
                const int x = i % W, yy = (i / W) % (ry + 2), ci = i / (W * (ry + 2));
                const int gy = y0 + yy - 1;
                sin[((size_t)ci * (rows + 2) + yy) * W + x] =
                    (gy >= 0 && gy < H) ? in[(((size_t)b * Ci + ci) * H + gy) * W + x] : 0.f;
            }
            for (int i = threadIdx.x; i < Co * ry * W; i += blockDim.x) {
                const int x = i % W, yy = (i / W) % ry, co = i / (W * ry);
                sd[((size_t)co * rows + yy) * W + x] = d[(((size_t)b * Co + co) * H + y0 + yy) * W + x];
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < kBwPer; ++j) {
                const int e = threadIdx.x + j * kBwThreads;
                if (e >= nent) continue;
                float sacc = acc[j];
                if (e < nw) {
                    const int kx = e % KW, ky = (e / KW) % KH, ci = (e / (KW * KH)) % Ci, co = e / (KW * KH * Ci);
                    for (int yy = 0; yy < ry; ++yy) {
                        const float *dr = sd + ((size_t)co * rows + yy) * W;
                        const float *ir = sin + ((size_t)ci * (rows + 2) + yy + ky) * W;
                        for (int x = 0; x < W; ++x) {
                            int xx = x + kx - 2;
                            xx += (xx < 0) ? W : 0;
                            xx -= (xx >= W) ? W : 0;
                            sacc = fmaf(dr[x], ir[xx], sacc);
                        }
                    }
                } else {
                    const int co = e - nw;
                    for (int yy = 0; yy < ry; ++yy) {
                        const float *dr = sd + ((size_t)co * rows + yy) * W;
                        for (int x = 0; x < W; ++x) sacc += dr[x];
                    }
                }
                acc[j] = sacc;
            }
        }
    }
#pragma unroll
    for (int j = 0; j < kBwPer; ++j) {
        const int e = threadIdx.x + j * kBwThreads;
        if (e < nent) part[(size_t)blockIdx.x * nent + e] = acc[j];
    }
}

__global__ void k_pn_sum_parts(const float *__restrict__ part, int nparts, int nw, int nent, float *__restrict__ dw,
                               float *__restrict__ db) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nent) return;
    float s = 0.f;
    for (int k = 0; k < nparts; ++k) s += part[(size_t)k * nent + e];
    if (e < nw)
        dw[e] = s;
    else
        db[e - nw] = s;
}

// Input gradient of a convolution through the ReLU of its input
// activation: one thread per input position (b, y, x) computes every input
// channel, the weights in shared memory; din = 0 where a <= 0.
__global__ void __launch_bounds__(256)
k_pn_conv_bwd_x(const float *__restrict__ d, int Co, const float *__restrict__ w, int Ci, int H, int W, int B,
                const float *__restrict__ a, float *__restrict__ din) {
    extern __shared__ float wsx[];  // [Co][Ci][KH*KW]
    const int nw = Co * Ci * KH * KW;
    for (int j = threadIdx.x; j < nw; j += blockDim.x) wsx[j] = w[j];
    __syncthreads();
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)B * H * W) return;
    const int x = (int)(i % W), y = (int)((i / W) % H), b = (int)(i / ((long long)W * H));
    float acc[kPnMaxCo];
#pragma unroll
    for (int ci = 0; ci < kPnMaxCo; ++ci) acc[ci] = 0.f;
    for (int co = 0; co < Co; ++co) {
        const float *src = d + ((size_t)b * Co + co) * H * W;
        float v[KH * KW];
        bool ok[KH];
#pragma unroll
        for (int ky = 0; ky < KH; ++ky) {
            const int yy = y - ky + 1;
            ok[ky] = yy >= 0 && yy < H;
#pragma unroll
            for (int kx = 0; kx < KW; ++kx) {
                int xx = x - kx + 2;
                xx += (xx < 0) ? W : 0;
                xx -= (xx >= W) ? W : 0;
                v[ky * KW + kx] = ok[ky] ? src[yy * W + xx] : 0.f;
            }
        }
#pragma unroll
        for (int ci = 0; ci < kPnMaxCo; ++ci) {
            if (ci >= Ci) continue;
            const float *wk = wsx + ((size_t)co * Ci + ci) * KH * KW;
            float s = acc[ci];
#pragma unroll
            for (int ky = 0; ky < KH; ++ky) {
                if (!ok[ky]) continue;
#pragma unroll
                for (int kx = 0; kx < KW; ++kx) s += wk[ky * KW + kx] * v[ky * KW + kx];
            }
            acc[ci] = s;
        }
    }
#pragma unroll
    for (int ci = 0; ci < kPnMaxCo; ++ci)
        if (ci < Ci) {
            const size_t o = (((size_t)b * Ci + ci) * H + y) * W + x;
            din[o] = a[o] > 0.f ? acc[ci] : 0.f;
        }
}

// Adam (Kingma & Ba 2015) with bias corrections c1 = 1 - beta1^t, c2 = 1 - beta2^t.
__global__ void k_pn_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                          float *__restrict__ v, long long n, float lr, float b1, float b2, float eps, float c1,
                          float c2) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// Top-M directions by logit and their softmax probabilities, one block per
// sample (M passes of a block arg-max over a shared copy).
__global__ void k_pn_topm(const float *__restrict__ logits, int N, int M, int *__restrict__ idx,
                          float *__restrict__ prob) {
    extern __shared__ float s_l[];
    __shared__ float sh[32];
    __shared__ float s_bv[32];
    __shared__ int s_bi[32];
    const int b = blockIdx.x;
    const float *l = logits + (size_t)b * N;
    float m = -3.4e38f;
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        s_l[n] = l[n];
        m = fmaxf(m, l[n]);
    }
    m = block_reduce(m, sh, true);
    float se = 0.f;
    for (int n = threadIdx.x; n < N; n += blockDim.x) se += expf(s_l[n] - m);
    se = block_reduce(se, sh, false);
    const float lse = m + logf(se);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    for (int k = 0; k < M; ++k) {
        float bv = -3.4e38f;
        int bi = 0x7fffffff;
        for (int n = threadIdx.x; n < N; n += blockDim.x)
            if (s_l[n] > bv || (s_l[n] == bv && n < bi)) {
                bv = s_l[n];
                bi = n;
            }
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > bv || (ov == bv && oi < bi)) {
                bv = ov;
                bi = oi;
            }
        }
        if (lane == 0) {
            s_bv[wid] = bv;
            s_bi[wid] = bi;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            float v0 = s_bv[0];
            int i0 = s_bi[0];
            for (int q = 1; q < nw; ++q)
                if (s_bv[q] > v0 || (s_bv[q] == v0 && s_bi[q] < i0)) {
                    v0 = s_bv[q];
                    i0 = s_bi[q];
                }
            if (i0 < 0 || i0 >= N) i0 = 0;  // every logit NaN
            idx[(size_t)b * M + k] = i0;
            prob[(size_t)b * M + k] = expf(v0 - lse);
            s_l[i0] = -3.4e38f;
        }
        __syncthreads();
    }
}

inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

cudaError_t pn_gen(const float *proj, int lda, const PixelRef *pix, int npix, const float *minv,
                   const float *ctf_pool, int full_npix, int n_pool, long long R, int NP, int ND, uint64_t seed,
                   int B, float *v, int *label, cudaStream_t st) {
    k_pn_gen<<<B, 128, 0, st>>>(proj, lda, pix, npix, minv, ctf_pool, full_npix, n_pool, R, NP, ND, seed, v, label);
    return cudaGetLastError();
}

cudaError_t pn_power(const float2 *fimg, int full_npix, const PixelRef *pix, int npix, const float *minv, int B,
                     float *v, cudaStream_t st) {
    k_pn_power<<<nblk((long long)B * npix, 256), 256, 0, st>>>(fimg, full_npix, pix, npix, minv, B, v);
    return cudaGetLastError();
}

cudaError_t pn_bin(const float *v, int npix, const int *bin, const float *inv_cnt, int nbins, int B, float *feat,
                   cudaStream_t st) {
    k_pn_bin<<<B, 128, sizeof(float) * nbins, st>>>(v, npix, bin, inv_cnt, nbins, feat);
    return cudaGetLastError();
}

cudaError_t pn_forward(const PnDims &d, const float *params, const float *feat, float *a1, float *a2, float *h,
                       float *logits, cudaStream_t st) {
    const int H = d.H, W = d.W, B = d.B;
    const float *w1 = params + d.o_w1, *b1 = params + d.o_b1, *w2 = params + d.o_w2, *b2 = params + d.o_b2;
    const float *w3 = params + d.o_w3, *b3 = params + d.o_b3;
    if (d.C1 > kPnMaxCo || d.C2 > kPnMaxCo) return cudaErrorInvalidValue;
    const size_t s1 = sizeof(float) * (d.C1 * 1 * KH * KW + d.C1), s2 = sizeof(float) * (d.C2 * d.C1 * KH * KW + d.C2);
    k_pn_conv_fwd<<<nblk((long long)B * H * W, 256), 256, s1, st>>>(feat, 1, w1, b1, d.C1, H, W, B, a1);
    k_pn_conv_fwd<<<nblk((long long)B * H * W, 256), 256, s2, st>>>(a1, d.C1, w2, b2, d.C2, H, W, B, a2);
    k_pn_pool<<<nblk((long long)B * d.C2 * H, 256), 256, 0, st>>>(a2, d.C2, H, W, B, h);
    k_pn_linear<<<nblk((long long)B * d.ND, 256), 256, 0, st>>>(h, d.C2 * H, w3, b3, d.ND, B, logits);
    return cudaGetLastError();
}

size_t pn_backward_scratch(const PnDims &d) {
    return (size_t)kBwParts * (d.C2 * d.C1 * KH * KW + d.C2);
}

// weight / bias gradients of one convolution (partials, then their sum)
static cudaError_t conv_bwd_w(const float *in, int Ci, const float *dd, int Co, int H, int W, int B, float *dw,
                              float *db, float *scratch, cudaStream_t st) {
    const int nent = Co * Ci * KH * KW + Co;
    if (nent > kBwThreads * kBwPer) return cudaErrorInvalidValue;
    // row tile: inputs with halo and output gradients within 96 KB
    const size_t cap = 96 * 1024 / sizeof(float);
    int rows = (int)std::min<long long>(H, ((long long)cap / W - 2 * Ci) / (Ci + Co));
    if (rows < 1) return cudaErrorInvalidValue;
    const size_t smem = sizeof(float) * ((size_t)Ci * (rows + 2) + (size_t)Co * rows) * W;
    static size_t attr = 0;
    if (smem > attr) {
        cudaError_t e = cudaFuncSetAttribute(k_pn_conv_bwd_w_part, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)std::max<size_t>(smem, 96 * 1024));
        if (e != cudaSuccess) return e;
        attr = std::max<size_t>(smem, 96 * 1024);
    }
    const int nparts = std::min(B, kBwParts);
    k_pn_conv_bwd_w_part<<<nparts, kBwThreads, smem, st>>>(in, Ci, dd, Co, H, W, B, rows, scratch);
    k_pn_sum_parts<<<nblk(nent, 256), 256, 0, st>>>(scratch, nparts, nent - Co, nent, dw, db);
    return cudaGetLastError();
}

cudaError_t pn_loss_backward(const PnDims &d, const float *params, const float *feat, const float *a1,
                             const float *a2, const float *h, const float *logits, const int *label,
                             const float *target, float *dl, float *loss, float *d2, float *d1, float *grad,
                             float *scratch, cudaStream_t st) {
    const int H = d.H, W = d.W, B = d.B, F = d.C2 * d.H;
    k_pn_xent<<<B, 256, 0, st>>>(logits, d.ND, label, target, B, dl, loss);
    k_pn_linear_bwd_w<<<nblk((long long)(F + 1) * d.ND, 256), 256, 0, st>>>(h, dl, F, d.ND, B, grad + d.o_w3,
                                                                             grad + d.o_b3);
    k_pn_linear_bwd_x<<<nblk((long long)B * F, 256), 256, 0, st>>>(dl, params + d.o_w3, F, d.ND, B, a2, W, d2);
    cudaError_t e = conv_bwd_w(a1, d.C1, d2, d.C2, H, W, B, grad + d.o_w2, grad + d.o_b2, scratch, st);
    if (e != cudaSuccess) return e;
    k_pn_conv_bwd_x<<<nblk((long long)B * H * W, 256), 256, sizeof(float) * d.C2 * d.C1 * KH * KW, st>>>(
        d2, d.C2, params + d.o_w2, d.C1, H, W, B, a1, d1);
    e = conv_bwd_w(feat, 1, d1, d.C1, H, W, B, grad + d.o_w1, grad + d.o_b1, scratch, st);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

cudaError_t pn_adam(float *p, const float *g, float *m, float *v, long long n, float lr, int t, cudaStream_t st) {
    const float b1 = 0.9f, b2 = 0.999f;
    const double p1 = std::pow((double)b1, (double)t), p2 = std::pow((double)b2, (double)t);
    k_pn_adam<<<nblk(n, 256), 256, 0, st>>>(p, g, m, v, n, lr, b1, b2, 1e-8f, (float)(1. - p1), (float)(1. - p2));
    return cudaGetLastError();
}

// Probability of each block of `dpb` consecutive directions under the
// tempered softmax softmax(logits / temperature): one CTA per particle.
__global__ void k_pn_block_probs(const float *__restrict__ logits, int N, int dpb, float inv_t,
                                 float *__restrict__ out) {
    __shared__ float sh[32];
    const int b = blockIdx.x;
    const float *l = logits + (size_t)b * N;
    float m = -3.4e38f;
    for (int n = threadIdx.x; n < N; n += blockDim.x) m = fmaxf(m, l[n] * inv_t);
    m = block_reduce(m, sh, true);
    float se = 0.f;
    for (int n = threadIdx.x; n < N; n += blockDim.x) se += expf(l[n] * inv_t - m);
    se = block_reduce(se, sh, false);
    const float inv_se = se > 0.f ? 1.f / se : 0.f;
    const int nb = N / dpb;
    for (int j = threadIdx.x; j < nb; j += blockDim.x) {
        float acc = 0.f;
        for (int q = 0; q < dpb; ++q) acc += expf(l[j * dpb + q] * inv_t - m);
        out[(size_t)b * nb + j] = acc * inv_se;
    }
}

cudaError_t pn_block_probs(const float *logits, int N, int dpb, float temperature, int B, float *out,
                           cudaStream_t st) {
    if (dpb < 1 || N % dpb != 0 || !(temperature > 0.f)) return cudaErrorInvalidValue;
    k_pn_block_probs<<<B, 256, 0, st>>>(logits, N, dpb, 1.f / temperature, out);
    return cudaGetLastError();
}

// The m most probable blocks of each particle (probability descending,
// lower index first among equals) and their summed probability: one warp
// per particle, m rounds of a warp arg-max over the block probabilities.
__global__ void k_pn_top_blocks(const float *__restrict__ probs, int nb, int m, int *__restrict__ idx,
                                float *__restrict__ mass) {
    extern __shared__ float pv[];  // [nb]
    const int b = blockIdx.x, lane = threadIdx.x;
    const float *pb = probs + (size_t)b * nb;
    for (int j = lane; j < nb; j += 32) pv[j] = pb[j];
    __syncwarp();
    float sum = 0.f;
    for (int k = 0; k < m; ++k) {
        float best = -1.f;
        int bi = 0x7fffffff;
        for (int j = lane; j < nb; j += 32) {
            const float v = pv[j];
            if (v > best || (v == best && j < bi)) {
                best = v;
                bi = j;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > best || (ov == best && oi < bi)) {
                best = ov;
                bi = oi;
            }
        }
        if (lane == 0) {
            idx[(size_t)b * m + k] = bi;
            pv[bi] = -2.f;  // taken
        }
        sum += best;
        __syncwarp();
    }
    if (lane == 0) mass[b] = sum;
}

cudaError_t pn_top_blocks(const float *probs, int nb, int m, int B, int *idx, float *mass, cudaStream_t st) {
    if (m < 1 || m > nb) return cudaErrorInvalidValue;
    k_pn_top_blocks<<<B, 32, sizeof(float) * nb, st>>>(probs, nb, m, idx, mass);
    return cudaGetLastError();
}

cudaError_t pn_topm(const float *logits, int N, int M, int B, int *idx, float *prob, cudaStream_t st) {
    k_pn_topm<<<B, 256, sizeof(float) * N, st>>>(logits, N, M, idx, prob);
    return cudaGetLastError();
}

}  // namespace gbr
