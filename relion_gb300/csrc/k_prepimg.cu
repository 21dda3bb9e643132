// k_prepimg.cu -- image preparation on the GPU: the E-step inputs of a batch
// of real-space particle images, as MlOptimiser::getFourierTransformsAndCtfs
// (src/ml_optimiser.cpp:5840-6753) prepares them for 2D single-particle
// data with --zero_mask (average background outside the mask), no CTF
// padding and no MTF / aberration corrections:
//   norm correction and integer shift by the rounded old offset (no wrap),
//   forward FFT / N^2 (cuFFT, FP32) of the unmasked and of the masked image,
//   window to the current size with CenterFFTbySign,
//   power spectrum and high-resolution power of the masked image,
//   CTF image on the full-box frequencies (CTF::getFftwImage).
#include <algorithm>

#include "gbr_internal.h"

#include <cufft.h>

namespace gbr {
namespace {

constexpr double kPiD = 3.14159265358979323846;

// Raised-cosine weight of the background at radius r (softMaskOutsideMap,
// src/mask.cpp:43-96): 0 inside `radius`, 1 beyond radius + width.
__device__ __forceinline__ double bg_weight(double r, double radius, double width) {
    if (r < radius) return 0.;
    const double rp = radius + width;
    if (r > rp) return 1.;
    return 0.5 + 0.5 * cos(kPiD * (rp - r) / width);
}

// Raised-cosine background weights of the N x N box, once per geometry.
__global__ void k_mask_weights(int N, double radius, double width, float *__restrict__ W) {
    const int h = N / 2;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N * N; i += gridDim.x * blockDim.x) {
        const int y = i / N - h, x = i % N - h;
        W[i] = (float)bg_weight(sqrt((double)(y * y + x * x)), radius, width);
    }
}

// A[p][y][x] = f_p in[p][y - dy_p][x - dx_p], 0 where the source is outside
// (translate with DONT_WRAP, src/transformations.h; V2(r) = V1(r - v)),
// together with the weighted background sums of the soft mask (sum w A,
// sum w): FP32 within a warp, FP64 across warps.
// Each thread takes kImgPer pixels one block-width apart, loads all of them
// before using any (memory-level parallelism), grid (N^2 / (256 kImgPer), n).
constexpr int kImgPer = 8;

__global__ void k_img_shift_bg(const float *__restrict__ in, int N, const int *__restrict__ shift,
                               const float *__restrict__ factor, const float *__restrict__ W,
                               float *__restrict__ A, double *__restrict__ sums) {
    const int p = blockIdx.y;
    const int dx = shift[2 * p], dy = shift[2 * p + 1];
    const float f = factor[p];
    const float *src = in + (size_t)p * N * N;
    float *dst = A + (size_t)p * N * N;
    const int NN = N * N, base = blockIdx.x * (blockDim.x * kImgPer) + threadIdx.x;
    const bool pow2 = (N & (N - 1)) == 0;
    const int lgN = __ffs(N) - 1;
    float v[kImgPer], wv[kImgPer];
#pragma unroll
    for (int k = 0; k < kImgPer; ++k) {
        const int i = base + k * blockDim.x;
        v[k] = 0.f;
        wv[k] = 0.f;
        if (i < NN) {
            const int y = pow2 ? (i >> lgN) : i / N, x = i - y * N;
            const int sy = y - dy, sx = x - dx;
            if (sy >= 0 && sy < N && sx >= 0 && sx < N) v[k] = src[(size_t)sy * N + sx];
            wv[k] = W[i];
        }
    }
    float fw = 0.f, fv = 0.f;
#pragma unroll
    for (int k = 0; k < kImgPer; ++k) {
        const int i = base + k * blockDim.x;
        if (i < NN) {
            const float val = f * v[k];
            dst[i] = val;
            fw += wv[k];
            fv = fmaf(wv[k], val, fv);
        }
    }
    // FP32 across the warp (a warp's 256 pixels), then each warp adds into
    // the particle's FP64 sums (L2 atomics): no block barrier and no serial
    // FP64 tail, so warps retire as their own loads complete
    for (int o = 16; o > 0; o >>= 1) {
        fw += __shfl_xor_sync(0xffffffffu, fw, o);
        fv += __shfl_xor_sync(0xffffffffu, fv, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&sums[2 * p], (double)fv);
        atomicAdd(&sums[2 * p + 1], (double)fw);
    }
}

__global__ void k_mask_apply(const float *__restrict__ A, int N, const float *__restrict__ W,
                             const double *__restrict__ sums, float *__restrict__ B) {
    const int p = blockIdx.y;
    const float *src = A + (size_t)p * N * N;
    float *dst = B + (size_t)p * N * N;
    const int NN = N * N, base = blockIdx.x * (blockDim.x * kImgPer) + threadIdx.x;
    float a[kImgPer], w[kImgPer];
#pragma unroll
    for (int k = 0; k < kImgPer; ++k) {
        const int i = base + k * blockDim.x;
        a[k] = i < NN ? src[i] : 0.f;
        w[k] = i < NN ? W[i] : 0.f;
    }
    // the background value, one FP64 division per block (FP64 is slow
    // here), while the pixel loads above are in flight
    __shared__ float s_b;
    if (threadIdx.x == 0) {
        const double sw = sums[2 * p + 1];
        s_b = (float)(sw > 0. ? sums[2 * p] / sw : 0.);
    }
    __syncthreads();
    const float b = s_b;
#pragma unroll
    for (int k = 0; k < kImgPer; ++k) {
        const int i = base + k * blockDim.x;
        if (i < NN) dst[i] = (1.f - w[k]) * a[k] + w[k] * b;
    }
}

// windowFourierTransform to `cur` (src/fftw.h:809-857) + CenterFFTbySign
// (src/fftw.h:390-403) + the 1/N^2 of the forward transform, of two
// transforms in one launch (blockIdx.z: F0 -> out0, F1 -> out1).
__global__ void k_window_center(const float2 *__restrict__ F0, const float2 *__restrict__ F1, int N, int cur,
                                float2 *__restrict__ out0, float2 *__restrict__ out1) {
    const float2 *__restrict__ F = blockIdx.z ? F1 : F0;
    float2 *__restrict__ out = blockIdx.z ? out1 : out0;
    const int p = blockIdx.y;
    const int X = cur / 2 + 1, half = N / 2 + 1;
    const float s = 1.f / ((float)N * (float)N);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < cur * X; e += gridDim.x * blockDim.x) {
        const int i = e / X, j = e - i * X;
        const int row = i < X ? i : N - cur + i;  // logical frequency i or i - cur
        float2 v = F[((size_t)p * N + row) * half + j];
        const float sg = ((i ^ j) & 1) ? -s : s;
        out[(size_t)p * cur * X + e] = make_float2(v.x * sg, v.y * sg);
    }
}

// Power spectrum per shell and power beyond the current size: blocks over
// row chunks of each particle, shells in shared memory, then global atomics
// (power and xi2 zeroed by the caller).
__global__ void k_img_spectrum(const float2 *__restrict__ F, int N, int cur, double *__restrict__ power,
                               double *__restrict__ xi2) {
    // FP32 partial sums per block (a chunk of N / gridDim.x rows: at most a
    // few hundred terms per shell), FP64 across blocks
    extern __shared__ float s_pw[];  // [half]
    const int p = blockIdx.y, half = N / 2 + 1;
    for (int i = threadIdx.x; i < half; i += blockDim.x) s_pw[i] = 0.f;
    __syncthreads();
    const float inv = 1.f / ((float)N * (float)N);
    // each thread takes runs of kRun consecutive x of one row and merges
    // neighbours that fall in the same shell before its shared atomic
    constexpr int kRun = 8;
    const int runs_per_row = (half + kRun - 1) / kRun;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < N * runs_per_row; q += gridDim.x * blockDim.x) {
        const int i = q / runs_per_row, j0 = (q - i * runs_per_row) * kRun;
        const int ip = i < half ? i : i - N;
        const float2 *row = F + ((size_t)p * N + i) * half;
        int cur_s = -1;
        float acc = 0.f;
        for (int j = j0; j < j0 + kRun && j < half; ++j) {
            const int ires = (int)floorf(sqrtf((float)(ip * ip + j * j)) + 0.5f);
            if (!(ires > 0 && ires < half && !(j == 0 && ip < 0))) continue;
            const float2 v = row[j];
            const float re = v.x * inv, im = v.y * inv;
            if (ires != cur_s) {
                if (cur_s >= 0) atomicAdd(&s_pw[cur_s], acc);
                cur_s = ires;
                acc = 0.f;
            }
            acc += re * re + im * im;
        }
        if (cur_s >= 0) atomicAdd(&s_pw[cur_s], acc);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < half; i += blockDim.x)
        if (s_pw[i] != 0.f) {
            atomicAdd(&power[(size_t)p * half + i], (double)s_pw[i]);
            if (i >= cur / 2 + 1) atomicAdd(&xi2[p], (double)s_pw[i]);
        }
}

// CTF::getCTF (src/ctf.h:184-256, damping on) with the constants of
// CTF::initialise (src/ctf.cpp:211-261), per particle: the astigmatic
// defocus form, K1 (wavelength), K2 (Cs), K3 (amplitude contrast), K4 (B
// factor), K5 (phase shift), scale.
struct CtfConst {
    double Axx, Axy, Ayy, K1, K2, K3, K4, K5, scale;
};

__device__ CtfConst ctf_const(const double *c, double kV, double Cs, double Q0) {
    const double defU = c[0], defV = c[1], defA = c[2], Bfac = c[3], scale = c[4], phase = c[5];
    const double local_Cs = Cs * 1e7, local_kV = kV * 1e3;
    const double rad_az = defA * kPiD / 180.;
    const double lambda = 12.2643247 / sqrt(local_kV * (1. + local_kV * 0.978466e-6));
    CtfConst k;
    k.K1 = kPiD / 2 * 2 * lambda;
    k.K2 = kPiD / 2 * local_Cs * lambda * lambda * lambda;
    k.K3 = atan(Q0 / sqrt(1 - Q0 * Q0));
    k.K4 = -Bfac / 4.;
    k.K5 = phase * kPiD / 180.;
    const double s = sin(rad_az), co = cos(rad_az);
    k.Axx = co * co * (-defU) + s * s * (-defV);
    k.Axy = co * s * (-defU) - s * co * (-defV);
    k.Ayy = s * s * (-defU) + co * co * (-defV);
    k.scale = scale;
    return k;
}

// Double-float arithmetic (Dekker, "A floating-point technique for extending
// the available precision", 1971): a value carried as an unevaluated FP32 sum
// hi + lo (~48 significant bits), with the error-free transformations of a
// sum (Knuth's two-sum) and of a product (by FMA).  The _rn intrinsics keep
// the compiler from contracting them.
struct DFloat {
    float hi, lo;
};

__device__ __forceinline__ DFloat df_split(double x) {
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
}

__device__ __forceinline__ DFloat two_sum(float a, float b) {
    const float s = __fadd_rn(a, b), v = __fadd_rn(s, -a);
    return {s, __fadd_rn(__fadd_rn(a, -__fadd_rn(s, -v)), __fadd_rn(b, -v))};
}

// a * f for an FP32 f
__device__ __forceinline__ DFloat df_mul_f(DFloat a, float f) {
    const float p = __fmul_rn(a.hi, f);
    return two_sum(p, fmaf(a.lo, f, fmaf(a.hi, f, -p)));
}

__device__ __forceinline__ DFloat df_add(DFloat a, DFloat b) {
    const DFloat s = two_sum(a.hi, b.hi);
    return two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

// 2 pi as an FP32 pair, for the reduction of the phase (Cody and Waite,
// "Software Manual for the Elementary Functions", 1980): g - n 2 pi with
// n 2pi_hi formed exactly by FMA.
constexpr float kTwoPiHi = (float)(2.0 * kPiD);
constexpr float kTwoPiLo = (float)(2.0 * kPiD - (double)kTwoPiHi);
constexpr float kInvTwoPiF = (float)(0.5 / kPiD);

// CTF image of the current size on the full-box frequencies
// (CTF::getFftwImage, src/ctf.cpp:314-450, no padding).  FP64 runs at a
// small fraction of the FP32 rate on this part, so:
//  * along a row (frequency y = ip s, x = j s, s = 1 / (N pixel)) the phase
//    is the polynomial in the column index j that it is,
//      gamma = K1 s^2 (Axx j^2 + 2 Axy ip j + Ayy ip^2) + K2 s^4 (j^2 + ip^2)^2 - K5 - K3
//            = C0 + B j + A2 j^2 + Q j^4,
//    with the particle's constants (K1 s^2 Axx, ..., K2 s^4) formed in FP64
//    once per block and the rows' coefficients from them in double-float
//    (an FP64 instruction occupies the FP64 pipe for tens of cycles whatever
//    the active lanes: the blocks are large so that this setup is rare);
//  * per pixel it is evaluated in double-float (j and j^2 are exact in FP32;
//    ~1e-14 relative, where FP64 gives ~1e-16) and reduced modulo 2 pi, all
//    in FP32 units;
//  * the sine of the reduced phase and the damping exponential are FP32
//    (|CTF| <= 1, error ~1e-7, the rounding of the reduced phase).
// A block covers kCtfRows rows of one particle.
constexpr int kCtfRows = 128;
__global__ void __launch_bounds__(256) k_ctf_image(const double *__restrict__ ctf, int N, int cur, double pixel,
                                                   double kV, double Cs, double Q0, float *__restrict__ out) {
    __shared__ DFloat s_c0[kCtfRows], s_b[kCtfRows], s_a2[kCtfRows];
    __shared__ float s_e0[kCtfRows];
    // particle constants: K1 s^2 Ayy, 2 K1 s^2 Axy, K1 s^2 Axx, K2 s^4, -K5 - K3
    __shared__ DFloat s_ayy, s_axy, s_axx, s_q, s_k53;
    __shared__ float s_e2, s_scale;
    const int p = blockIdx.y, X = cur / 2 + 1, r0 = blockIdx.x * kCtfRows;
    const int nr = min(kCtfRows, cur - r0);
    if (threadIdx.x == 0) {
        const CtfConst k = ctf_const(ctf + (size_t)p * 6, kV, Cs, Q0);
        const double sc = 1. / ((double)N * pixel), s2 = sc * sc, k1 = k.K1 * s2;
        s_ayy = df_split(k1 * k.Ayy);
        s_axy = df_split(2.0 * k1 * k.Axy);
        s_axx = df_split(k1 * k.Axx);
        s_q = df_split(k.K2 * s2 * s2);
        s_k53 = df_split(-k.K5 - k.K3);
        s_e2 = (float)(k.K4 * s2);
        s_scale = (float)k.scale;
    }
    __syncthreads();
    if (threadIdx.x < nr) {
        // C0 = K1 s^2 Ayy ip^2 + Q ip^4 - K5 - K3, B = 2 K1 s^2 Axy ip,
        // A2 = K1 s^2 Axx + 2 Q ip^2 (ip and ip^2 exact in FP32)
        const int i = r0 + threadIdx.x;
        const float ip = (float)(i < X ? i : i - cur), ip2 = ip * ip;
        const DFloat qip2 = df_mul_f(s_q, ip2);
        s_c0[threadIdx.x] = df_add(df_add(df_mul_f(s_ayy, ip2), df_mul_f(qip2, ip2)), s_k53);
        s_b[threadIdx.x] = df_mul_f(s_axy, ip);
        s_a2[threadIdx.x] = df_add(s_axx, df_mul_f(qip2, 2.f));
        s_e0[threadIdx.x] = s_e2 * ip2;
    }
    __syncthreads();
    const DFloat q = s_q;
    const float e2 = s_e2, scale = s_scale;
    float *o = out + (size_t)p * cur * X + (size_t)r0 * X;
    for (int e = threadIdx.x; e < nr * X; e += blockDim.x) {
        const int il = e / X, j = e - il * X;
        const float jf = (float)j, tf = (float)(j * j);  // exact: j < 2^12
        const DFloat g = df_add(df_mul_f(df_add(df_mul_f(q, tf), s_a2[il]), tf), df_add(df_mul_f(s_b[il], jf), s_c0[il]));
        const float n = rintf(g.hi * kInvTwoPiF);
        const float pn = __fmul_rn(n, kTwoPiHi), pe = fmaf(n, kTwoPiHi, -pn);
        const float rg = __fadd_rn(__fadd_rn(g.hi, -pn), __fadd_rn(__fadd_rn(g.lo, -pe), -__fmul_rn(n, kTwoPiLo)));
        const float arg = fmaf(e2, tf, s_e0[il]);
        float r = -sinf(rg) * expf(arg) * scale;
        if (fabsf(r) < 1e-8f) r = (r < 0.f ? -1.f : 1.f) * 1e-8f;
        o[e] = r;
    }
}

}  // namespace

cudaError_t launch_prepare_images(const PrepImagesArgs &a, cudaStream_t st) {
    const int n = a.n, N = a.N, cur = a.cur;
    if (n <= 0) return cudaSuccess;
    // (the CTF image takes j^2 exact in FP32: j = cur / 2 below 2^12)
    if (N <= 0 || (N & 1) || cur <= 0 || (cur & 1) || cur > N || cur / 2 >= 4096) return cudaErrorInvalidValue;
    const int X = cur / 2 + 1, half = N / 2 + 1;
    const dim3 gimg((unsigned)((N * N + 256 * kImgPer - 1) / (256 * kImgPer)), (unsigned)n);
    if (a.mask_fresh) k_mask_weights<<<(N * N + 255) / 256, 256, 0, st>>>(N, a.mask_radius, a.mask_width, a.W);
    cudaError_t e = cudaMemsetAsync(a.bg, 0, sizeof(double) * 2 * n, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(a.power, 0, sizeof(double) * (size_t)n * half, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(a.xi2, 0, sizeof(double) * n, st);
    if (e != cudaSuccess) return e;
    k_img_shift_bg<<<gimg, 256, 0, st>>>(a.images, N, a.shift, a.factor, a.W, a.A, a.bg);
    k_mask_apply<<<gimg, 256, 0, st>>>(a.A, N, a.W, a.bg, a.B);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    cufftHandle plan = (cufftHandle)a.fft_plan;
    if (cufftSetStream(plan, st) != CUFFT_SUCCESS) return cudaErrorUnknown;
    if (cufftExecR2C(plan, a.A, reinterpret_cast<cufftComplex *>(a.FA)) != CUFFT_SUCCESS) return cudaErrorUnknown;
    if (cufftExecR2C(plan, a.B, reinterpret_cast<cufftComplex *>(a.FB)) != CUFFT_SUCCESS) return cudaErrorUnknown;
    const dim3 gw((unsigned)((cur * X + 255) / 256), (unsigned)n, 2u);
    k_window_center<<<gw, 256, 0, st>>>(a.FA, a.FB, N, cur, a.fimg_nomask, a.fimg);
    // spectrum: 8 row chunks per particle (few FP64 atomics per shell)
    const dim3 gs((unsigned)std::min(8, std::max(1, N / 32)), (unsigned)n);
    if (cur < N) k_img_spectrum<<<gs, 256, sizeof(float) * half, st>>>(a.FB, N, cur, a.power, a.xi2);
    // CTF: blocks of kCtfRows rows of each particle
    k_ctf_image<<<dim3((unsigned)((cur + kCtfRows - 1) / kCtfRows), (unsigned)n), 256, 0, st>>>(
        a.ctf, N, cur, a.pixel, a.kV, a.Cs, a.Q0, a.fctf);
    return cudaGetLastError();
}

int make_fft_plan(int N, int batch, long long *plan_out) {
    cufftHandle plan;
    int dims[2] = {N, N};
    if (cufftPlanMany(&plan, 2, dims, nullptr, 1, 0, nullptr, 1, 0, CUFFT_R2C, batch) != CUFFT_SUCCESS) return -1;
    *plan_out = (long long)plan;
    return 0;
}

void destroy_fft_plan(long long plan) {
    if (plan >= 0) cufftDestroy((cufftHandle)plan);
}

}  // namespace gbr
