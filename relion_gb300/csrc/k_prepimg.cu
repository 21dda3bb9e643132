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
#include "gbr_internal.h"

#include <cufft.h>

namespace gbr {
namespace {

constexpr double kPiD = 3.14159265358979323846;

// A[p][y][x] = f_p in[p][y - dy_p][x - dx_p], 0 where the source is outside
// (translate with DONT_WRAP, src/transformations.h; V2(r) = V1(r - v)).
__global__ void k_img_shift(const float *__restrict__ in, int N, const int *__restrict__ shift,
                            const float *__restrict__ factor, float *__restrict__ A) {
    const int p = blockIdx.y;
    const int dx = shift[2 * p], dy = shift[2 * p + 1];
    const float f = factor[p];
    const float *src = in + (size_t)p * N * N;
    float *dst = A + (size_t)p * N * N;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N * N; i += gridDim.x * blockDim.x) {
        const int y = i / N, x = i - y * N;
        const int sy = y - dy, sx = x - dx;
        dst[i] = (sy >= 0 && sy < N && sx >= 0 && sx < N) ? f * src[(size_t)sy * N + sx] : 0.f;
    }
}

// Raised-cosine weight of the background at radius r (softMaskOutsideMap,
// src/mask.cpp:43-96): 0 inside `radius`, 1 beyond radius + width.
__device__ __forceinline__ double bg_weight(double r, double radius, double width) {
    if (r < radius) return 0.;
    const double rp = radius + width;
    if (r > rp) return 1.;
    return 0.5 + 0.5 * cos(kPiD * (rp - r) / width);
}

// Average background value per particle (one block per particle).
__global__ void k_mask_bg(const float *__restrict__ A, int N, double radius, double width, double *__restrict__ bg) {
    __shared__ double s_sum[32], s_w[32];
    const int p = blockIdx.x, h = N / 2;
    const float *img = A + (size_t)p * N * N;
    double sw = 0., sv = 0.;
    for (int i = threadIdx.x; i < N * N; i += blockDim.x) {
        const int y = i / N - h, x = i % N - h;
        const double w = bg_weight(sqrt((double)(y * y + x * x)), radius, width);
        sw += w;
        sv += w * (double)img[i];
    }
    for (int o = 16; o > 0; o >>= 1) {
        sw += __shfl_xor_sync(0xffffffffu, sw, o);
        sv += __shfl_xor_sync(0xffffffffu, sv, o);
    }
    if ((threadIdx.x & 31) == 0) {
        s_w[threadIdx.x >> 5] = sw;
        s_sum[threadIdx.x >> 5] = sv;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tw = 0., tv = 0.;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            tw += s_w[i];
            tv += s_sum[i];
        }
        bg[p] = tw > 0. ? tv / tw : 0.;
    }
}

__global__ void k_mask_apply(const float *__restrict__ A, int N, double radius, double width,
                             const double *__restrict__ bg, float *__restrict__ B) {
    const int p = blockIdx.y, h = N / 2;
    const float *src = A + (size_t)p * N * N;
    float *dst = B + (size_t)p * N * N;
    const double b = bg[p];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N * N; i += gridDim.x * blockDim.x) {
        const int y = i / N - h, x = i % N - h;
        const double w = bg_weight(sqrt((double)(y * y + x * x)), radius, width);
        dst[i] = (float)((1. - w) * (double)src[i] + w * b);
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

// Power spectrum per shell and power beyond the current size (one block per
// particle, shells in shared memory).
__global__ void k_img_spectrum(const float2 *__restrict__ F, int N, int cur, double *__restrict__ power,
                               double *__restrict__ xi2) {
    extern __shared__ double s_pw[];  // [half]
    const int p = blockIdx.x, half = N / 2 + 1;
    for (int i = threadIdx.x; i < half; i += blockDim.x) s_pw[i] = 0.;
    __syncthreads();
    const double inv = 1. / ((double)N * (double)N);
    if (cur < N) {
        for (int e = threadIdx.x; e < N * half; e += blockDim.x) {
            const int i = e / half, j = e - i * half;
            const int ip = i < half ? i : i - N;
            const int ires = (int)floor(sqrt((double)(ip * ip + j * j)) + 0.5);
            if (ires > 0 && ires < half && !(j == 0 && ip < 0)) {
                const float2 v = F[(size_t)p * N * half + e];
                const double re = (double)v.x * inv, im = (double)v.y * inv;
                atomicAdd(&s_pw[ires], re * re + im * im);
            }
        }
    }
    __syncthreads();
    double hx = 0.;
    for (int i = threadIdx.x; i < half; i += blockDim.x) {
        power[(size_t)p * half + i] = s_pw[i];
        if (i >= cur / 2 + 1) hx += s_pw[i];
    }
    for (int o = 16; o > 0; o >>= 1) hx += __shfl_xor_sync(0xffffffffu, hx, o);
    __shared__ double s_h[32];
    if ((threadIdx.x & 31) == 0) s_h[threadIdx.x >> 5] = hx;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += s_h[i];
        xi2[p] = t;
    }
}

// CTF::getCTF (src/ctf.h:184-256, damping on) at spatial frequency (X, Y) in
// 1/Angstrom, with the constants of CTF::initialise (src/ctf.cpp:211-261).
__device__ double ctf_at(const double *c, double kV, double Cs, double Q0, double X, double Y) {
    const double defU = c[0], defV = c[1], defA = c[2], Bfac = c[3], scale = c[4], phase = c[5];
    const double local_Cs = Cs * 1e7, local_kV = kV * 1e3;
    const double rad_az = defA * kPiD / 180.;
    const double lambda = 12.2643247 / sqrt(local_kV * (1. + local_kV * 0.978466e-6));
    const double K1 = kPiD / 2 * 2 * lambda;
    const double K2 = kPiD / 2 * local_Cs * lambda * lambda * lambda;
    const double K3 = atan(Q0 / sqrt(1 - Q0 * Q0));
    const double K4 = -Bfac / 4.;
    const double K5 = phase * kPiD / 180.;
    const double s = sin(rad_az), co = cos(rad_az);
    const double Axx = co * co * (-defU) + s * s * (-defV);
    const double Axy = co * s * (-defU) - s * co * (-defV);
    const double Ayy = s * s * (-defU) + co * co * (-defV);
    const double u2 = X * X + Y * Y, u4 = u2 * u2;
    const double gamma = K1 * (Axx * X * X + 2.0 * Axy * X * Y + Ayy * Y * Y) + K2 * u4 - K5 - K3;
    double r = -sin(gamma) * exp(K4 * u2) * scale;
    if (fabs(r) < 1e-8) r = (r < 0 ? -1. : 1.) * 1e-8;
    return r;
}

// CTF image of the current size on the full-box frequencies
// (CTF::getFftwImage, src/ctf.cpp:314-450, no padding).
__global__ void k_ctf_image(const double *__restrict__ ctf, int N, int cur, double pixel, double kV, double Cs,
                            double Q0, float *__restrict__ out) {
    const int p = blockIdx.y, X = cur / 2 + 1;
    const double xs = (double)N * pixel;
    const double *c = ctf + (size_t)p * 6;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < cur * X; e += gridDim.x * blockDim.x) {
        const int i = e / X, j = e - i * X;
        const int ip = i < X ? i : i - cur;
        out[(size_t)p * cur * X + e] = (float)ctf_at(c, kV, Cs, Q0, (double)j / xs, (double)ip / xs);
    }
}

}  // namespace

cudaError_t launch_prepare_images(const PrepImagesArgs &a, cudaStream_t st) {
    const int n = a.n, N = a.N, cur = a.cur;
    if (n <= 0) return cudaSuccess;
    if (N <= 0 || (N & 1) || cur <= 0 || (cur & 1) || cur > N) return cudaErrorInvalidValue;
    const int X = cur / 2 + 1, half = N / 2 + 1;
    const dim3 gimg((unsigned)((N * N + 255) / 256 < 1024 ? (N * N + 255) / 256 : 1024), (unsigned)n);
    k_img_shift<<<gimg, 256, 0, st>>>(a.images, N, a.shift, a.factor, a.A);
    k_mask_bg<<<n, 256, 0, st>>>(a.A, N, a.mask_radius, a.mask_width, a.bg);
    k_mask_apply<<<gimg, 256, 0, st>>>(a.A, N, a.mask_radius, a.mask_width, a.bg, a.B);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    cufftHandle plan = (cufftHandle)a.fft_plan;
    if (cufftSetStream(plan, st) != CUFFT_SUCCESS) return cudaErrorUnknown;
    if (cufftExecR2C(plan, a.A, reinterpret_cast<cufftComplex *>(a.FA)) != CUFFT_SUCCESS) return cudaErrorUnknown;
    if (cufftExecR2C(plan, a.B, reinterpret_cast<cufftComplex *>(a.FB)) != CUFFT_SUCCESS) return cudaErrorUnknown;
    const dim3 gw((unsigned)((cur * X + 255) / 256), (unsigned)n);
    k_window_center<<<gw, 256, 0, st>>>(a.FA, N, cur, a.fimg_nomask);
    k_window_center<<<gw, 256, 0, st>>>(a.FB, N, cur, a.fimg);
    k_img_spectrum<<<n, 256, sizeof(double) * half, st>>>(a.FB, N, cur, a.power, a.xi2);
    k_ctf_image<<<gw, 256, 0, st>>>(a.ctf, N, cur, a.pixel, a.kV, a.Cs, a.Q0, a.fctf);
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
