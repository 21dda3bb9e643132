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
// sum w): a few pixels per thread in FP32, FP64 across threads and blocks.
// Each thread takes kImgPer pixels one block-width apart, loads all of them
// before using any (memory-level parallelism), grid (N^2 / (256 kImgPer), n).
constexpr int kImgPer = 8;

__global__ void k_img_shift_bg(const float *__restrict__ in, int N, const int *__restrict__ shift,
                               const float *__restrict__ factor, const float *__restrict__ W,
                               float *__restrict__ A, double *__restrict__ sums) {
    __shared__ double s_v[32], s_w[32];
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
    double sw = fw, sv = fv;
    for (int o = 16; o > 0; o >>= 1) {
        sw += __shfl_xor_sync(0xffffffffu, sw, o);
        sv += __shfl_xor_sync(0xffffffffu, sv, o);
    }
    if ((threadIdx.x & 31) == 0) {
        s_w[threadIdx.x >> 5] = sw;
        s_v[threadIdx.x >> 5] = sv;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tw = 0., tv = 0.;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            tw += s_w[i];
            tv += s_v[i];
        }
        atomicAdd(&sums[2 * p], tv);
        atomicAdd(&sums[2 * p + 1], tw);
    }
}

__global__ void k_mask_apply(const float *__restrict__ A, int N, const float *__restrict__ W,
                             const double *__restrict__ sums, float *__restrict__ B) {
    const int p = blockIdx.y;
    const float *src = A + (size_t)p * N * N;
    float *dst = B + (size_t)p * N * N;
    // the background value, one FP64 division per block (FP64 is slow here)
    __shared__ float s_b;
    if (threadIdx.x == 0) {
        const double sw = sums[2 * p + 1];
        s_b = (float)(sw > 0. ? sums[2 * p] / sw : 0.);
    }
    __syncthreads();
    const float b = s_b;
    const int NN = N * N, base = blockIdx.x * (blockDim.x * kImgPer) + threadIdx.x;
    float a[kImgPer], w[kImgPer];
#pragma unroll
    for (int k = 0; k < kImgPer; ++k) {
        const int i = base + k * blockDim.x;
        a[k] = i < NN ? src[i] : 0.f;
        w[k] = i < NN ? W[i] : 0.f;
    }
#pragma unroll
    for (int k = 0; k < kImgPer; ++k) {
        const int i = base + k * blockDim.x;
        if (i < NN) dst[i] = (1.f - w[k]) * a[k] + w[k] * b;
    }
}

// windowFourierTransform to `cur` (src/fftw.h:809-857) + CenterFFTbySign
// (src/fftw.h:390-403) + the 1/N^2 of the forward transform.
__global__ void k_window_center(const float2 *__restrict__ F, int N, int cur, float2 *__restrict__ out) {
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

// CTF image of the current size on the full-box frequencies
// (CTF::getFftwImage, src/ctf.cpp:314-450, no padding).  The phase gamma is
// formed in FP64 and reduced modulo 2 pi there; the sine and the damping
// exponential of the reduced values are FP32 (|CTF| <= 1, error ~1e-7).
__global__ void k_ctf_image(const double *__restrict__ ctf, int N, int cur, double pixel, double kV, double Cs,
                            double Q0, float *__restrict__ out) {
    __shared__ CtfConst sk;
    const int p = blockIdx.y, X = cur / 2 + 1;
    if (threadIdx.x == 0) sk = ctf_const(ctf + (size_t)p * 6, kV, Cs, Q0);
    __syncthreads();
    const CtfConst k = sk;
    const double inv_xs = 1. / ((double)N * pixel);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < cur * X; e += gridDim.x * blockDim.x) {
        const int i = e / X, j = e - i * X;
        const int ip = i < X ? i : i - cur;
        const double x = (double)j * inv_xs, y = (double)ip * inv_xs;
        const double u2 = x * x + y * y;
        double g = k.K1 * (k.Axx * x * x + 2.0 * k.Axy * x * y + k.Ayy * y * y) + k.K2 * u2 * u2 - k.K5 - k.K3;
        g -= 2. * kPiD * rint(g * (0.5 / kPiD));
        float r = -sinf((float)g) * expf((float)(k.K4 * u2)) * (float)k.scale;
        if (fabsf(r) < 1e-8f) r = (r < 0.f ? -1.f : 1.f) * 1e-8f;
        out[(size_t)p * cur * X + e] = r;
    }
}

}  // namespace

cudaError_t launch_prepare_images(const PrepImagesArgs &a, cudaStream_t st) {
    const int n = a.n, N = a.N, cur = a.cur;
    if (n <= 0) return cudaSuccess;
    if (N <= 0 || (N & 1) || cur <= 0 || (cur & 1) || cur > N) return cudaErrorInvalidValue;
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
    const dim3 gw((unsigned)((cur * X + 255) / 256), (unsigned)n);
    k_window_center<<<gw, 256, 0, st>>>(a.FA, N, cur, a.fimg_nomask);
    k_window_center<<<gw, 256, 0, st>>>(a.FB, N, cur, a.fimg);
    // spectrum: 8 row chunks per particle (few FP64 atomics per shell)
    const dim3 gs((unsigned)std::min(8, std::max(1, N / 32)), (unsigned)n);
    if (cur < N) k_img_spectrum<<<gs, 256, sizeof(float) * half, st>>>(a.FB, N, cur, a.power, a.xi2);
    // CTF: the particle's constants formed once per block, blocks over its pixels
    k_ctf_image<<<dim3((unsigned)((cur * X + 255) / 256), (unsigned)n), 256, 0, st>>>(a.ctf, N, cur, a.pixel, a.kV,
                                                                                   a.Cs, a.Q0, a.fctf);
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
