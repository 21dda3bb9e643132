// Reconstruction side of an iteration on the device, in FP64 with cuFFT
// double-precision transforms (the reference computes it in double):
//   BackProjector::enforceHermitianSymmetry  src/backprojector.cpp:2148-2165
//   BackProjector::updateSSNRarrays          src/backprojector.cpp:1041-1204
//   BackProjector::reconstruct               src/backprojector.cpp:1379-1872
//     (convoluteBlobRealSpace :2483-2528, windowToOridimRealSpace :2530-2670,
//      softMaskOutsideMap src/mask.cpp:43-96, griddingCorrect src/projector.cpp:595-628)
//   Projector::computeFourierTransformMap    src/projector.cpp:116-593
//   getFSC                                   src/fftw.cpp:481-525
// Every pass is one grid-stride kernel over an FFTW half grid or a real
// box; the shell sums use per-block shared-memory histograms flushed with
// FP64 atomics.  Transforms are in place (real rows padded to 2 (N/2+1)).
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <array>
#include <map>
#include <type_traits>
#include <string>
#include <vector>

#include "gbr_internal.h"

namespace gbr {

namespace {

const double kPi = 3.14159265358979323846;
const int kBlobTab = 10000;  // TabFtBlob entries (BackProjector constructor)
const int kThreads = 256;

// FFTW half layout of an N^dim real array: [Z][N][N/2+1], Z = N (3D) or 1 (2D)
struct Half {
    int N, Z, Y, X, dim;
    __host__ __device__ long long size() const { return (long long)Z * Y * X; }
    __host__ __device__ int rowp() const { return 2 * X; }  // padded real row (in-place transforms)
    __device__ void at(long long n, int &k, int &i, int &j) const {
        if (n <= 0x7fffffffLL) {  // 32-bit divisions (several times cheaper than 64-bit)
            const unsigned u = (unsigned)n, t = u / (unsigned)X;
            j = (int)(u - t * (unsigned)X);
            i = (int)(t % (unsigned)Y);
            k = (int)(t / (unsigned)Y);
            return;
        }
        j = (int)(n % X);
        const long long t = n / X;
        i = (int)(t % Y);
        k = (int)(t / Y);
    }
    // FOR_ALL_ELEMENTS_IN_FFTW_TRANSFORM (src/fftw.h:99-102)
    __device__ int kp(int k) const { return (k < X) ? k : k - Z; }
    __device__ int ip(int i) const { return (i < X) ? i : i - Y; }
};

Half make_half(int N, int dim) { return Half{N, dim == 3 ? N : 1, N, N / 2 + 1, dim}; }

// element types of the transformed arrays: FP64 (the reference's precision)
// or FP32 (GB300's FP64 rate is a small fraction of its FP32 rate); weights,
// shell sums and the final map stay FP64 either way
template <class R> struct Cx;
template <> struct Cx<double> { typedef double2 T; };
template <> struct Cx<float> { typedef float2 T; };
template <class R> __device__ __forceinline__ typename Cx<R>::T cmake(double a, double b);
template <> __device__ __forceinline__ double2 cmake<double>(double a, double b) { return make_double2(a, b); }
template <> __device__ __forceinline__ float2 cmake<float>(double a, double b) {
    return make_float2((float)a, (float)b);
}

// n -> (z, y, x) of a [.][B][A] array, 32-bit divisions when n fits
__device__ __forceinline__ void decode3(long long n, int A, int B, int &z, int &y, int &x) {
    if (n <= 0x7fffffffLL) {
        const unsigned u = (unsigned)n, t = u / (unsigned)A;
        x = (int)(u - t * (unsigned)A);
        y = (int)(t % (unsigned)B);
        z = (int)(t / (unsigned)B);
        return;
    }
    x = (int)(n % A);
    const long long t = n / A;
    y = (int)(t % B);
    z = (int)(t / B);
}

__host__ __device__ __forceinline__ int d_round(double x) { return (x > 0) ? (int)(x + 0.5) : (int)(x - 0.5); }

// logical (k, i, j) of a projector / backprojector array, x from 0
__device__ __forceinline__ long long cidx(const VolGeom &g, int k, int i, int j) {
    return ((long long)(k - g.zinit) * g.ydim + (i - g.yinit)) * g.xdim + j;
}

// MAP term of BackProjector::reconstruct (:1454-1493)
struct MapTerm {
    const double *tau2;
    double ovc_fudge;  // oversampling_correction * tau2_fudge
    double pad;
    int minres, on;
    const int *iround;  // ROUND(sqrt(r2) / pad) by r2
};

// Per-r2 tables, built once on the host in double precision (GB300's FP64
// rate makes a sqrt / sin / cos per voxel the bottleneck of these passes):
// shell indices ROUND(sqrt(r2) / p) and FLOOR(sqrt(r2) / p), and for the
// real-space box the gridding correction 1 / sinc^2 and the soft-mask
// weight (< 0 inside the radius, > 1.5 beyond the cosine edge).
struct RealTab {
    const double *inv_sinc2;
    const double *rc;
};

// decenter(weight) (src/projector.h:249-260) plus the MAP term
__device__ __forceinline__ double fweight_at(const double *weight, const VolGeom &g, int kp, int ip, int jp, int r2,
                                             int max_r2, const MapTerm &m) {
    double fw = (r2 <= max_r2) ? weight[cidx(g, kp, ip, jp)] : 0.;
    if (m.on && r2 < max_r2) {
        const int ires = m.iround[r2];
        const double t = m.tau2[ires];
        const double inv = (t > 0.) ? 1. / (m.ovc_fudge * t) : ((fw > 1e-20) ? 1. / (0.001 * fw) : 0.);
        if (ires >= m.minres) fw = fw + inv;
    }
    return fw;
}

int grid_for(long long n) {
    long long b = (n + kThreads - 1) / kThreads;
    return (int)std::max<long long>(1, std::min<long long>(b, 152LL * 8));
}

// ---------------------------------------------------------------------------
// enforceHermitianSymmetry: every (iz, iy) pair with its mirror once
__global__ void k_hermitian(double2 *data, double *weight, VolGeom g) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= (long long)g.zdim * g.ydim) return;
    const int iz = g.zinit + (int)(n / g.ydim), iy = g.yinit + (int)(n % g.ydim);
    if (iy < ((iz < 0) ? 0 : 1)) return;
    const long long a = cidx(g, iz, iy, 0), b = cidx(g, -iz, -iy, 0);
    const double2 da = data[a], db = data[b];
    const double2 s = make_double2(da.x + db.x, da.y - db.y);
    data[a] = s;
    data[b] = make_double2(s.x, -s.y);
    const double w = weight[a] + weight[b];
    weight[a] = w;
    weight[b] = w;
}

// updateSSNRarrays, pass 0: sigma2 and counter; pass 1: data_vs_prior,
// coverage and counter with the final tau2.  sums [3][ns]
__global__ void k_ssnr(const double *weight, VolGeom g, int max_r2, const int *iround, double ovc, int pass,
                       const double *tau2, double ovc_fudge, int upd, int ns, double *sums) {
    extern __shared__ double sh[];
    for (int b = threadIdx.x; b < 3 * ns; b += blockDim.x) sh[b] = 0.;
    __syncthreads();
    const long long nvox = (long long)g.zdim * g.ydim * g.xdim;
    for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < nvox;
         n += (long long)gridDim.x * blockDim.x) {
        int k, i, j;
        decode3(n, g.xdim, g.ydim, k, i, j);
        i += g.yinit;
        k += g.zinit;
        const int r2 = k * k + i * i + j * j;
        if (r2 >= max_r2) continue;
        const int ires = iround[r2];
        const double w = weight[n];
        if (pass == 0) {
            atomicAdd(&sh[ires], ovc * w);
        } else {
            const double tt = tau2[ires];
            const double invtau2 = (tt > 0.) ? 1. / (ovc_fudge * tt) : 1. / (0.001 * w);
            const double ratio = w / invtau2;
            if (!upd) atomicAdd(&sh[ires], ratio);
            if (ratio >= 1.) atomicAdd(&sh[2 * ns + ires], 1.);
        }
        atomicAdd(&sh[ns + ires], 1.);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < 3 * ns; b += blockDim.x)
        if (sh[b] != 0.) atomicAdd(&sums[b], sh[b]);
}

// skip-gridding branch: radial sums of Fweight (FLOOR shells) [2][r_max]
__global__ void k_radavg(const double *weight, VolGeom g, Half h, int max_r2, int round_max_r2, MapTerm m,
                         const int *ifloor, int r_max, double *sums) {
    extern __shared__ double sh[];
    for (int b = threadIdx.x; b < 2 * r_max; b += blockDim.x) sh[b] = 0.;
    __syncthreads();
    // runs of kRunR consecutive elements per thread, neighbours of one shell
    // summed before the shared-memory atomic
    constexpr int kRunR = 8;
    for (long long n0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * kRunR; n0 < h.size();
         n0 += (long long)gridDim.x * blockDim.x * kRunR) {
        int cur = -1;
        double acc = 0., cnt = 0.;
        for (int q = 0; q < kRunR && n0 + q < h.size(); ++q) {
            int k, i, j;
            h.at(n0 + q, k, i, j);
            const int kp = h.kp(k), ip = h.ip(i);
            const int r2 = kp * kp + ip * ip + j * j;
            if (r2 >= round_max_r2) continue;
            const int ires = ifloor[r2];
            if (ires != cur) {
                if (cur >= 0) {
                    atomicAdd(&sh[cur], acc);
                    atomicAdd(&sh[r_max + cur], cnt);
                }
                cur = ires;
                acc = 0.;
                cnt = 0.;
            }
            acc += fweight_at(weight, g, kp, ip, j, r2, max_r2, m);
            cnt += 1.;
        }
        if (cur >= 0) {
            atomicAdd(&sh[cur], acc);
            atomicAdd(&sh[r_max + cur], cnt);
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < 2 * r_max; b += blockDim.x)
        if (sh[b] != 0.) atomicAdd(&sums[b], sh[b]);
}

// Final Fourier array of the reconstruction, written straight into the
// padded box of windowToOridimRealSpace: windowFourierTransform
// (src/fftw.h:809-857) from the odd grid `hin` to the even grid `hout`, the
// skip-gridding division by max(Fweight, radavg) (:1499-1560) or the
// gridding weights (:1683-1694), and CenterFFTbySign (src/fftw.h:389-402).
// mode 0: skip gridding (sums = radial sums [2][r_max]); mode 1: gridding
// (fn = Fnewweight on hin, data divided by normalise).
template <class R>
__global__ void k_window(const double2 *data, const double *weight, VolGeom g, Half hin, Half hout, int max_r2,
                         MapTerm m, const int *ifloor, int mode, const double *sums, int r_max, const double *fn,
                         double normalise, typename Cx<R>::T *out, int *err) {
    extern __shared__ double ra[];
    if (mode == 0) {
        for (int b = threadIdx.x; b < r_max; b += blockDim.x) {
            const double v = sums[b], c = sums[r_max + b];
            if (c > 0. || v > 0.) {
                ra[b] = v / (1000. * c);
            } else {
                ra[b] = 0.;
                atomicOr(err, 1);  // "zeros in counter or radavg_weight"
            }
        }
        __syncthreads();
    }
    const bool upsize = hout.X > hin.X;
    const int wr2 = (hin.X - 1) * (hin.X - 1);
    for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < hout.size();
         n += (long long)gridDim.x * blockDim.x) {
        int k, i, j;
        hout.at(n, k, i, j);
        const int kp = hout.kp(k), ip = hout.ip(i);
        const int r2 = kp * kp + ip * ip + j * j;
        double2 v = make_double2(0., 0.);
        if ((!upsize || r2 <= wr2) && r2 <= max_r2) {
            v = data[cidx(g, kp, ip, j)];
            if (mode == 0) {
                const double fw = fweight_at(weight, g, kp, ip, j, r2, max_r2, m);
                const int ires = ifloor[r2];
                const double w = fmax(fw, ra[(ires < r_max) ? ires : (r_max - 1)]);
                if (w != 0.) v = make_double2(v.x / w, v.y / w);
            } else {
                const int ki = kp < 0 ? kp + hin.Z : kp, ii = ip < 0 ? ip + hin.Y : ip;
                const double f = fn[((long long)ki * hin.Y + ii) * hin.X + j];
                v = make_double2(v.x / normalise * f, v.y / normalise * f);
            }
        }
        if ((k ^ i ^ j) & 1) v = make_double2(-v.x, -v.y);
        // self-conjugate elements (every index 0 or N/2) are real: the
        // half-complex inverse ignores their imaginary parts (FFTW's c2r does;
        // cuFFT's FP32 C2R does not)
        if ((k == 0 || 2 * k == hout.Z) && (i == 0 || 2 * i == hout.Y) && (j == 0 || 2 * j == hout.N)) v.y = 0.;
        out[n] = cmake<R>(v.x, v.y);
    }
}

// gridding branch initialisation (:1571-1598): Fweight / normalise, the
// Fnewweight indicator and the first convolution input Fnewweight * Fweight
template <class R>
__global__ void k_grid_init(const double *weight, VolGeom g, Half h, int max_r2, MapTerm m, double normalise,
                            double *fw, double *fn, typename Cx<R>::T *C) {
    for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < h.size();
         n += (long long)gridDim.x * blockDim.x) {
        int k, i, j;
        h.at(n, k, i, j);
        const int kp = h.kp(k), ip = h.ip(i);
        const int r2 = kp * kp + ip * ip + j * j;
        const double w = fweight_at(weight, g, kp, ip, j, r2, max_r2, m) / normalise;
        const double f = (r2 < max_r2) ? 1. : 0.;
        fw[n] = w;
        fn[n] = f;
        C[n] = cmake<R>(f * w, 0.);
    }
}

// convoluteBlobRealSpace (:2483-2528) on the real array of an in-place
// transform: multiply by the blob's Fourier value over its value at 0, and
// by 1 / N^dim, the normalisation of the forward transform that follows
template <class R>
__global__ void k_blob(R *M, Half h, const double *tab, double sampling, double inv_norm, double inv_scale,
                       double ori_pad) {
    const int padh = h.N / 2;
    const long long total = (long long)h.Z * h.Y * h.N;
    for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < total;
         n += (long long)gridDim.x * blockDim.x) {
        int k, i, j;
        decode3(n, h.N, h.Y, k, i, j);
        const int kp = (h.dim == 3) ? ((k < padh) ? k : k - h.N) : 0;
        const int ip = (i < padh) ? i : i - h.N, jp = (j < padh) ? j : j - h.N;
        const double rval = sqrt((double)(kp * kp + ip * ip + jp * jp)) / ori_pad;
        const int idx = (int)(fabs(rval) / sampling);
        const double b = (idx >= kBlobTab) ? 0. : tab[idx];
        R &e = M[((long long)k * h.Y + i) * h.rowp() + j];
        e = (R)((double)e * (b * inv_norm) * inv_scale);
    }
}

// one gridding iteration's division (:1633-1649) and the next input
template <class R>
__global__ void k_grid_update(typename Cx<R>::T *C, const double *fw, double *fn, Half h, int max_r2) {
    for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < h.size();
         n += (long long)gridDim.x * blockDim.x) {
        int k, i, j;
        h.at(n, k, i, j);
        const int kp = h.kp(k), ip = h.ip(i);
        double f = fn[n];
        if (kp * kp + ip * ip + j * j < max_r2) {
            const double cx = C[n].x, cy = C[n].y;
            f /= fmax(1e-6, sqrt(cx * cx + cy * cy));
            fn[n] = f;
        }
        C[n] = cmake<R>(f * fw[n], 0.);
    }
}

// window the padded real box to ori (centred), divide by normfft and sum the
// background of softMaskOutsideMap (radius ori/2, cosine width 3): bg [2]
template <class R>
__global__ void k_crop_bg(const R *M, int No, int rowp, int ori, int dim, double normfft, RealTab tab, double *vol,
                          double *bg) {
    __shared__ double s_sum[kThreads / 32], s_bg[kThreads / 32];
    const int h = ori / 2, off = No / 2 - h;
    const long long total = (long long)(dim == 3 ? ori : 1) * ori * ori;
    double sum = 0., sbg = 0.;
    for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < total;
         n += (long long)gridDim.x * blockDim.x) {
        int z, y, x;
        decode3(n, ori, ori, z, y, x);
        const int zo = dim == 3 ? z + off : 0;
        const double v = (double)M[((long long)zo * No + (y + off)) * rowp + (x + off)] / normfft;
        vol[n] = v;
        const int k = dim == 3 ? z - h : 0, i = y - h, j = x - h;
        const double rc = tab.rc[k * k + i * i + j * j];
        if (rc < 0.) continue;
        if (rc > 1.5) {
            sum += 1.;
            sbg += v;
        } else {
            sum += rc;
            sbg += rc * v;
        }
    }
    for (int o = 16; o; o >>= 1) {
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        sbg += __shfl_xor_sync(0xffffffffu, sbg, o);
    }
    if ((threadIdx.x & 31) == 0) {
        s_sum[threadIdx.x >> 5] = sum;
        s_bg[threadIdx.x >> 5] = sbg;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0., b = 0.;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            a += s_sum[w];
            b += s_bg[w];
        }
        atomicAdd(&bg[0], a);
        atomicAdd(&bg[1], b);
    }
}

// apply softMaskOutsideMap with the background average, then
// griddingCorrect (trilinear: divide by sinc^2 for r > 0)
__global__ void k_mask_gridcorr(double *vol, int ori, int dim, RealTab tab, const double *bg) {
    const int h = ori / 2;
    const long long total = (long long)(dim == 3 ? ori : 1) * ori * ori;
    const double avg = bg[1] / bg[0];
    for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < total;
         n += (long long)gridDim.x * blockDim.x) {
        int z, y, x;
        decode3(n, ori, ori, z, y, x);
        const int k = dim == 3 ? z - h : 0, i = y - h, j = x - h;
        const int r2 = k * k + i * i + j * j;
        const double rc = tab.rc[r2];
        double v = vol[n];
        if (rc >= 0.) v = rc > 1.5 ? avg : (1 - rc) * v + rc * avg;
        vol[n] = v * tab.inv_sinc2[r2];
    }
}

// computeFourierTransformMap: gridding pre-correction and zero padding into
// the real rows of an in-place transform of size No
template <class R>
__global__ void k_pad_map(const double *vol, int ori, int dim, int No, int rowp, const double *inv_sinc2,
                          R *M) {
    const int h = ori / 2, ho = No / 2;
    const long long total = (long long)(dim == 3 ? No : 1) * No * rowp;
    for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < total;
         n += (long long)gridDim.x * blockDim.x) {
        int z, y, x;
        decode3(n, rowp, No, z, y, x);
        const int k = dim == 3 ? z - ho : 0, i = y - ho, j = x - ho;
        double v = 0.;
        if (x < No && k >= -h && k < ori - h && i >= -h && i < ori - h && j >= -h && j < ori - h) {
            v = vol[((long long)(dim == 3 ? k + h : 0) * ori + (i + h)) * ori + (j + h)];
            if (inv_sinc2) v *= inv_sinc2[k * k + i * i + j * j];
        }
        M[n] = (R)v;
    }
}

// computeFourierTransformMap (:505-536): normalise, CenterFFTbySign, keep
// r2 <= max_r2 in the projector layout, radial power [2][ns]
template <class R>
__global__ void k_fill_projector(const typename Cx<R>::T *F, Half h, VolGeom pg, int max_r2, int min_r2, double nreal,
                                 double normfft, const int *iround, int ns, float2 *proj, double *power) {
    extern __shared__ double sh[];
    for (int b = threadIdx.x; b < 2 * ns; b += blockDim.x) sh[b] = 0.;
    __syncthreads();
    constexpr int kRunF = 8;  // consecutive elements per thread, one shell summed before its atomic
    for (long long n0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * kRunF; n0 < h.size();
         n0 += (long long)gridDim.x * blockDim.x * kRunF) {
        int cur = -1;
        double acc = 0., cnt = 0.;
        for (int q = 0; q < kRunF && n0 + q < h.size(); ++q) {
            const long long n = n0 + q;
            int k, i, j;
            h.at(n, k, i, j);
            const int kp = h.kp(k), ip = h.ip(i);
            const int r2 = kp * kp + ip * ip + j * j;
            if (r2 > max_r2) continue;
            double2 v = make_double2((double)F[n].x / nreal, (double)F[n].y / nreal);
            if ((k ^ i ^ j) & 1) v = make_double2(-v.x, -v.y);
            v = make_double2(v.x * normfft, v.y * normfft);
            const int ires = iround[r2];
            if (ires != cur) {
                if (cur >= 0) {
                    atomicAdd(&sh[cur], acc);
                    atomicAdd(&sh[ns + cur], cnt);
                }
                cur = ires;
                acc = 0.;
                cnt = 0.;
            }
            acc += (v.x * v.x + v.y * v.y) / 2.;
            cnt += 1.;
            if (r2 <= min_r2) v = make_double2(0., 0.);
            proj[cidx(pg, kp, ip, j)] = make_float2((float)v.x, (float)v.y);
        }
        if (cur >= 0) {
            atomicAdd(&sh[cur], acc);
            atomicAdd(&sh[ns + cur], cnt);
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < 2 * ns; b += blockDim.x)
        if (sh[b] != 0.) atomicAdd(&power[b], sh[b]);
}

// getFSC shell sums [3][X]: Re(conj z1 z2), |z1|^2, |z2|^2
template <class R>
__global__ void k_fsc(const typename Cx<R>::T *F1, const typename Cx<R>::T *F2, Half h, double nreal, const int *iround1,
                      double *sums) {
    extern __shared__ double sh[];
    for (int b = threadIdx.x; b < 3 * h.X; b += blockDim.x) sh[b] = 0.;
    __syncthreads();
    for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < h.size();
         n += (long long)gridDim.x * blockDim.x) {
        int k, i, j;
        h.at(n, k, i, j);
        const int kp = h.kp(k), ip = h.ip(i);
        const int idx = iround1[kp * kp + ip * ip + j * j];
        if (idx >= h.X) continue;
        const double2 z1 = make_double2((double)F1[n].x / nreal, (double)F1[n].y / nreal);
        const double2 z2 = make_double2((double)F2[n].x / nreal, (double)F2[n].y / nreal);
        atomicAdd(&sh[idx], z1.x * z2.x + z1.y * z2.y);
        const double a1 = sqrt(z1.x * z1.x + z1.y * z1.y), a2 = sqrt(z2.x * z2.x + z2.y * z2.y);
        atomicAdd(&sh[h.X + idx], a1 * a1);
        atomicAdd(&sh[2 * h.X + idx], a2 * a2);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < 3 * h.X; b += blockDim.x)
        if (sh[b] != 0.) atomicAdd(&sums[b], sh[b]);
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
#define RC_CUDA(expr)                                                                       \
    do {                                                                                    \
        cudaError_t e_ = (expr);                                                            \
        if (e_ != cudaSuccess) {                                                            \
            set_error_text(std::string(#expr) + ": " + cudaGetErrorString(e_));             \
            return e_ == cudaErrorMemoryAllocation ? kErrOom : kErrCuda;                    \
        }                                                                                   \
    } while (0)
#define RC_FFT(expr)                                                                        \
    do {                                                                                    \
        cufftResult r_ = (expr);                                                            \
        if (r_ != CUFFT_SUCCESS) {                                                          \
            set_error_text(std::string(#expr) + ": cuFFT error " + std::to_string((int)r_)); \
            return r_ == CUFFT_ALLOC_FAILED ? kErrOom : kErrCuda;                           \
        }                                                                                   \
    } while (0)

namespace {
const int kErrInvalid = -1, kErrCuda = -2, kErrOom = -3, kErrNumerical = -4;

int fail_recon(int st, const std::string &msg) {
    set_error_text(msg);
    return st;
}

// device scratch that grows to the largest request
struct Scratch {
    void *p = nullptr;
    size_t bytes = 0;
    ~Scratch() {
        if (p) cudaFree(p);
    }
    cudaError_t reserve(size_t b) {
        if (b <= bytes && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(b, 16));
        if (e == cudaSuccess) bytes = std::max<size_t>(b, 16);
        return e;
    }
    template <class T>
    T *as() const { return static_cast<T *>(p); }
};

// TabFtBlob of the order-0 Kaiser-Bessel blob, radius 1.9 * 2, alpha 15
// (BackProjector defaults, src/backprojector.h:80-115), divided by its value
// at 0; kaiser_Fourier_value (src/funcs.cpp:232-255) with I_{3/2} / J_{3/2}
// written in closed form (spherical Bessel functions).
std::vector<double> blob_table() {
    const double a = 1.9 * 2., alpha = 15., sampling = 0.5 / kBlobTab;
    auto f = [&](double w) {
        const double s2 = 2. * kPi * a * w, sigma = std::sqrt(std::fabs(alpha * alpha - s2 * s2));
        double b;
        if (sigma == 0.) return 0.;
        if (s2 > alpha) b = std::sqrt(2 / (kPi * sigma)) * (std::sin(sigma) / sigma - std::cos(sigma));
        else b = std::sqrt(2 / (kPi * sigma)) * (std::cosh(sigma) - std::sinh(sigma) / sigma);
        return b / std::pow(sigma, 1.5);
    };
    std::vector<double> t(kBlobTab);
    for (int i = 0; i < kBlobTab; ++i) t[i] = f(i * sampling);
    return t;
}
}  // namespace

struct ReconWork {
    Scratch c1, c2, fw, fn, vol, small, tab;
    std::map<long long, cufftHandle> plans;
    std::map<std::array<int, 4>, Scratch> tabs;  // per-r2 tables by (kind, a, b, entries)
    bool have_tab = false;
    bool fp32 = false;  // transforms in FP32 instead of FP64
    ~ReconWork() {
        for (auto &kv : plans) cufftDestroy(kv.second);
    }
    // plan of an in-place N^dim transform of the given type, cached
    int plan(int N, int dim, cufftType type, cufftHandle *out) {
        const long long key = ((long long)N << 16) | (dim << 12) | (int)type;
        auto it = plans.find(key);
        if (it != plans.end()) {
            *out = it->second;
            return 0;
        }
        cufftHandle h;
        if (dim == 3) RC_FFT(cufftPlan3d(&h, N, N, N, type));
        else RC_FFT(cufftPlan2d(&h, N, N, type));
        plans[key] = h;
        *out = h;
        return 0;
    }
};

namespace {
// in-place inverse (half -> real, unscaled) and forward (real -> half) transforms
template <class R>
int exec_inv(ReconWork *w, int N, int dim, void *buf) {
    const bool f = std::is_same<R, float>::value;
    cufftHandle h;
    const int st = w->plan(N, dim, f ? CUFFT_C2R : CUFFT_Z2D, &h);
    if (st) return st;
    if (f) RC_FFT(cufftExecC2R(h, static_cast<cufftComplex *>(buf), static_cast<cufftReal *>(buf)));
    else RC_FFT(cufftExecZ2D(h, static_cast<cufftDoubleComplex *>(buf), static_cast<cufftDoubleReal *>(buf)));
    return 0;
}
template <class R>
int exec_fwd(ReconWork *w, int N, int dim, void *buf) {
    const bool f = std::is_same<R, float>::value;
    cufftHandle h;
    const int st = w->plan(N, dim, f ? CUFFT_R2C : CUFFT_D2Z, &h);
    if (st) return st;
    if (f) RC_FFT(cufftExecR2C(h, static_cast<cufftReal *>(buf), static_cast<cufftComplex *>(buf)));
    else RC_FFT(cufftExecD2Z(h, static_cast<cufftDoubleReal *>(buf), static_cast<cufftDoubleComplex *>(buf)));
    return 0;
}
}  // namespace

void recon_set_fp32(ReconWork *w, int fp32) { w->fp32 = fp32 != 0; }

namespace {
// Device table of n entries of type T built by fill(r2) on the host, cached.
template <class T, class F>
const T *cached_table(ReconWork *w, int kind, int a, int b, int n, F fill, int &st) {
    const std::array<int, 4> key{kind, a, b, n};
    auto it = w->tabs.find(key);
    if (it != w->tabs.end()) return it->second.as<T>();
    std::vector<T> h((size_t)n);
    for (int r2 = 0; r2 < n; ++r2) h[(size_t)r2] = fill(r2);
    Scratch &sc = w->tabs[key];
    cudaError_t e = sc.reserve(sizeof(T) * (size_t)n);
    if (e == cudaSuccess) e = cudaMemcpy(sc.p, h.data(), sizeof(T) * (size_t)n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        set_error_text(std::string("reconstruction table: ") + cudaGetErrorString(e));
        st = e == cudaErrorMemoryAllocation ? kErrOom : kErrCuda;
        w->tabs.erase(key);
        return nullptr;
    }
    return sc.as<T>();
}

// ROUND(sqrt(r2) / p) (floor_mode 0) or FLOOR(sqrt(r2) / p) for r2 < n
const int *shell_table(ReconWork *w, int p, int n, int floor_mode, int &st) {
    return cached_table<int>(w, floor_mode ? 1 : 0, p, 0, n, [&](int r2) {
        const double x = std::sqrt((double)r2) / p;
        return floor_mode ? (int)x : d_round(x);
    }, st);
}

// gridding correction and soft-mask weights of the real box (ori, pad)
RealTab real_tables(ReconWork *w, int ori, int pad, int &st) {
    const int n = 3 * (ori / 2) * (ori / 2) + 1;
    RealTab t{};
    t.inv_sinc2 = cached_table<double>(w, 2, ori, pad, n, [&](int r2) {
        const double r = std::sqrt((double)r2);
        if (!(r > 0.)) return 1.;
        const double rval = r / ((double)ori * pad);
        const double sinc = std::sin(kPi * rval) / (kPi * rval);
        return 1. / (sinc * sinc);
    }, st);
    if (!t.inv_sinc2) return t;
    t.rc = cached_table<double>(w, 3, ori, 0, n, [&](int r2) {
        const double r = std::sqrt((double)r2), radius = (double)ori / 2., radius_p = radius + 3.;
        if (r < radius) return -1.;
        if (r > radius_p) return 2.;
        return 0.5 + 0.5 * std::cos(kPi * (radius_p - r) / 3.);
    }, st);
    return t;
}
}  // namespace

ReconWork *recon_work_create() { return new ReconWork(); }
void recon_work_destroy(ReconWork *w) { delete w; }

VolGeom projector_geometry(int ori, int dim, int pad, int current_size) {
    int r_max = current_size < 0 ? ori / 2 : current_size / 2;
    r_max = std::min(r_max, ori / 2);
    const int ps = 2 * (d_round((double)pad * r_max) + 1) + 1;
    return dim == 3 ? VolGeom{ps / 2 + 1, ps, ps, -(ps / 2), -(ps / 2), r_max, pad, 3}
                    : VolGeom{ps / 2 + 1, ps, 1, -(ps / 2), 0, r_max, pad, 2};
}

int recon_symmetrise(double2 *data, double *weight, const VolGeom &g) {
    const long long n = (long long)g.zdim * g.ydim;
    k_hermitian<<<(unsigned)((n + kThreads - 1) / kThreads), kThreads>>>(data, weight, g);
    RC_CUDA(cudaGetLastError());
    RC_CUDA(cudaDeviceSynchronize());
    return 0;
}

int recon_update_ssnr(ReconWork *w, const double *weight, const VolGeom &g, int ori, double tau2_fudge,
                      double *tau2_io, double *sigma2_out, double *dvp_out, double *cov_out, const double *fsc,
                      int upd, int whole) {
    const int ns = ori / 2 + 1;
    const double pad = g.pad, ovc = g.dim == 3 ? pad * pad * pad : pad * pad;
    const int mr = d_round(g.r_max * pad), max_r2 = mr * mr;
    const long long nvox = (long long)g.zdim * g.ydim * g.xdim;
    RC_CUDA(w->small.reserve(sizeof(double) * 4 * ns));
    double *sums = w->small.as<double>(), *tau2_d = sums + 3 * ns;
    std::vector<double> h(3 * ns);
    const size_t smem = sizeof(double) * 3 * ns;
    RC_CUDA(cudaMemset(sums, 0, smem));
    int tst = 0;
    const int *iround = shell_table(w, g.pad, mr * mr + 1, 0, tst);
    if (!iround) return tst;
    k_ssnr<<<grid_for(nvox), kThreads, smem>>>(weight, g, max_r2, iround, ovc, 0, nullptr, 0., upd, ns, sums);
    RC_CUDA(cudaGetLastError());
    RC_CUDA(cudaMemcpy(h.data(), sums, smem, cudaMemcpyDeviceToHost));
    std::vector<double> sigma2(ns), tau2(tau2_io, tau2_io + ns), dvp(ns, 0.), cov(ns, 0.);
    for (int i = 0; i < ns; ++i) {
        if (h[i] > 1e-20) sigma2[i] = h[ns + i] / h[i];
        else if (h[i] == 0) sigma2[i] = 0.;
        else return fail_recon(kErrNumerical, "updateSSNRarrays: unexpectedly small, yet non-zero sigma2 value");
    }
    if (upd)
        for (int i = 0; i < ns; ++i) {
            double f = std::max(0.001, fsc[i]);
            if (whole) f = std::sqrt(2. * f / (f + 1.));
            f = std::min(0.999, f);
            double ssnr = f / (1. - f);
            ssnr *= tau2_fudge;
            tau2[i] = ssnr * sigma2[i];
            dvp[i] = ssnr;
        }
    // shells reached by voxels inside r_max must not hold a negative tau2
    const int top = std::min(ns - 1, d_round(std::sqrt((double)std::max(0, max_r2 - 1)) / pad));
    for (int i = 0; i <= top; ++i)
        if (tau2[i] < 0.) return fail_recon(kErrNumerical, "updateSSNRarrays: negative tau2 spectrum");
    RC_CUDA(cudaMemcpy(tau2_d, tau2.data(), sizeof(double) * ns, cudaMemcpyHostToDevice));
    RC_CUDA(cudaMemset(sums, 0, smem));
    k_ssnr<<<grid_for(nvox), kThreads, smem>>>(weight, g, max_r2, iround, ovc, 1, tau2_d, ovc * tau2_fudge, upd, ns,
                                                sums);
    RC_CUDA(cudaGetLastError());
    RC_CUDA(cudaMemcpy(h.data(), sums, smem, cudaMemcpyDeviceToHost));
    for (int i = 0; i < ns; ++i) {
        const double cnt = h[ns + i];
        if (!upd) dvp[i] = (i > g.r_max) ? 0. : (cnt < 0.001 ? 999. : h[i] / cnt);
        cov[i] = cnt > 0. ? h[2 * ns + i] / cnt : h[2 * ns + i];
    }
    std::copy(tau2.begin(), tau2.end(), tau2_io);
    if (sigma2_out) std::copy(sigma2.begin(), sigma2.end(), sigma2_out);
    if (dvp_out) std::copy(dvp.begin(), dvp.end(), dvp_out);
    if (cov_out) std::copy(cov.begin(), cov.end(), cov_out);
    return 0;
}

namespace {

template <class R>
int reconstruct_impl(ReconWork *w, const double2 *data, const double *weight, const VolGeom &g, int ori,
                     const ReconParams &p, const double *tau2_host, double *vol_host) {
    typedef typename Cx<R>::T C2;
    const int dim = g.dim, N = g.ydim, r_max = g.r_max;
    const double pad = g.pad;
    if (r_max < 1 || N % 2 == 0) return fail_recon(kErrInvalid, "reconstruct: bad backprojector geometry");
    const bool grid = !p.skip_gridding && p.max_iter_preweight > 0;
    if (grid && p.normalise == 0.) return fail_recon(kErrInvalid, "reconstruct: normalise must be non-zero");
    const Half hin = make_half(N, dim);
    int No = d_round(pad * ori);
    No += No % 2;
    const Half hout = make_half(No, dim);
    const int mr = d_round(r_max * pad), max_r2 = mr * mr;
    const double ovc = dim == 3 ? pad * pad * pad : pad * pad;
    const int ns = ori / 2 + 1;
    // small scratch: tau2 [ns], radial sums [2 r_max], background [2], error flag
    RC_CUDA(w->small.reserve(sizeof(double) * (ns + 2 * r_max + 2 + 1)));
    double *tau2_d = w->small.as<double>(), *sums = tau2_d + ns, *bg = sums + 2 * r_max;
    int *err = reinterpret_cast<int *>(bg + 2);
    RC_CUDA(cudaMemset(sums, 0, sizeof(double) * (2 * r_max + 2 + 1)));
    if (p.do_map) {
        if (!tau2_host) return fail_recon(kErrInvalid, "reconstruct: do_map needs tau2");
        RC_CUDA(cudaMemcpy(tau2_d, tau2_host, sizeof(double) * ns, cudaMemcpyHostToDevice));
    }
    int tst = 0;
    const int *iround = shell_table(w, g.pad, max_r2 + 1, 0, tst);
    const int *ifloor = iround ? shell_table(w, g.pad, max_r2 + 1, 1, tst) : nullptr;
    const RealTab rtab = ifloor ? real_tables(w, ori, g.pad, tst) : RealTab{};
    if (!rtab.rc) return tst;
    const MapTerm m{tau2_d, ovc * p.tau2_fudge, pad, p.minres_map, p.do_map ? 1 : 0, iround};
    RC_CUDA(w->c1.reserve(sizeof(C2) * hout.size()));
    C2 *Fo = w->c1.as<C2>();
    if (!grid) {
        const int rm2 = d_round(r_max * pad * r_max * pad);
        k_radavg<<<grid_for(hin.size() / 8 + 1), kThreads, sizeof(double) * 2 * r_max>>>(
            weight, g, hin, max_r2, rm2, m, ifloor, r_max, sums);
        RC_CUDA(cudaGetLastError());
        k_window<R><<<grid_for(hout.size()), kThreads, sizeof(double) * r_max>>>(
            data, weight, g, hin, hout, max_r2, m, ifloor, 0, sums, r_max, nullptr, 1., Fo, err);
        RC_CUDA(cudaGetLastError());
    } else {
        RC_CUDA(w->c2.reserve(sizeof(C2) * hin.size()));
        RC_CUDA(w->fw.reserve(sizeof(double) * hin.size()));
        RC_CUDA(w->fn.reserve(sizeof(double) * hin.size()));
        C2 *C = w->c2.as<C2>();
        double *fw = w->fw.as<double>(), *fn = w->fn.as<double>();
        if (!w->have_tab) {
            const std::vector<double> t = blob_table();
            RC_CUDA(w->tab.reserve(sizeof(double) * t.size()));
            RC_CUDA(cudaMemcpy(w->tab.p, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice));
            w->have_tab = true;
        }
        double tab0 = 0.;
        RC_CUDA(cudaMemcpy(&tab0, w->tab.p, sizeof(double), cudaMemcpyDeviceToHost));
        k_grid_init<R><<<grid_for(hin.size()), kThreads>>>(weight, g, hin, max_r2, m, p.normalise, fw, fn, C);
        RC_CUDA(cudaGetLastError());
        const double nreal = (double)hin.Z * hin.Y * hin.N;
        for (int it = 0; it < p.max_iter_preweight; ++it) {
            int st = exec_inv<R>(w, N, dim, C);
            if (st) return st;
            k_blob<R><<<grid_for((long long)hin.Z * hin.Y * hin.N), kThreads>>>(
                reinterpret_cast<R *>(C), hin, w->tab.as<double>(), 0.5 / kBlobTab, 1. / tab0, 1. / nreal,
                (double)ori * pad);
            RC_CUDA(cudaGetLastError());
            st = exec_fwd<R>(w, N, dim, C);
            if (st) return st;
            k_grid_update<R><<<grid_for(hin.size()), kThreads>>>(C, fw, fn, hin, max_r2);
            RC_CUDA(cudaGetLastError());
        }
        k_window<R><<<grid_for(hout.size()), kThreads, 0>>>(data, weight, g, hin, hout, max_r2, m, ifloor, 1, sums,
                                                             r_max, fn, p.normalise, Fo, err);
        RC_CUDA(cudaGetLastError());
    }
    int st = exec_inv<R>(w, No, dim, Fo);
    if (st) return st;
    const long long nv = (long long)(dim == 3 ? ori : 1) * ori * ori;
    RC_CUDA(w->vol.reserve(sizeof(double) * nv));
    double *vol = w->vol.as<double>();
    const double normfft = dim == 3 ? pad * pad * pad * ori : pad * pad;
    k_crop_bg<R><<<grid_for(nv), kThreads>>>(reinterpret_cast<const R *>(Fo), No, hout.rowp(), ori, dim, normfft, rtab,
                                             vol, bg);
    RC_CUDA(cudaGetLastError());
    k_mask_gridcorr<<<grid_for(nv), kThreads>>>(vol, ori, dim, rtab, bg);
    RC_CUDA(cudaGetLastError());
    int herr = 0;
    RC_CUDA(cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) return fail_recon(kErrNumerical, "reconstruct: zeros in counter or radavg_weight");
    if (vol_host) RC_CUDA(cudaMemcpy(vol_host, vol, sizeof(double) * nv, cudaMemcpyDeviceToHost));
    return 0;
}

template <class R>
int projector_impl(ReconWork *w, const double *vol_host, int ori, int dim, int pad, const VolGeom &pg,
                   int do_gridding, int min_ires, float2 *proj, double *power_host) {
    typedef typename Cx<R>::T C2;
    int No = d_round((double)pad * ori);
    No += No % 2;
    const Half ho = make_half(No, dim);
    const long long nv = (long long)(dim == 3 ? ori : 1) * ori * ori;
    const int ns = ori / 2 + 1;
    if (vol_host) {
        RC_CUDA(w->vol.reserve(sizeof(double) * nv));
        RC_CUDA(cudaMemcpy(w->vol.p, vol_host, sizeof(double) * nv, cudaMemcpyHostToDevice));
    } else if (w->vol.bytes < sizeof(double) * nv) {
        return fail_recon(kErrInvalid, "no device-resident map of this size");
    }
    RC_CUDA(w->c1.reserve(sizeof(C2) * ho.size()));
    C2 *F = w->c1.as<C2>();
    const long long nreal_p = (long long)ho.Z * ho.Y * ho.rowp();
    int tst = 0;
    const RealTab rtab = real_tables(w, ori, pad, tst);
    if (!rtab.rc) return tst;
    k_pad_map<R><<<grid_for(nreal_p), kThreads>>>(w->vol.as<double>(), ori, dim, No, ho.rowp(),
                                                  do_gridding ? rtab.inv_sinc2 : nullptr, reinterpret_cast<R *>(F));
    RC_CUDA(cudaGetLastError());
    int st = exec_fwd<R>(w, No, dim, F);
    if (st) return st;
    RC_CUDA(cudaMemset(proj, 0, sizeof(float2) * (size_t)pg.xdim * pg.ydim * pg.zdim));
    RC_CUDA(w->small.reserve(sizeof(double) * 2 * ns));
    double *sums = w->small.as<double>();
    RC_CUDA(cudaMemset(sums, 0, sizeof(double) * 2 * ns));
    const int mr = d_round(pg.r_max * (double)pad), max_r2 = mr * mr;
    const int mn = d_round(min_ires * (double)pad), min_r2 = min_ires > 0 ? mn * mn : -1;
    const double normfft = dim == 3 ? (double)pad * pad * pad * ori : (double)pad * pad;
    const double nreal = (double)ho.Z * ho.Y * ho.N;
    const int *iround = shell_table(w, pad, max_r2 + 1, 0, tst);
    if (!iround) return tst;
    k_fill_projector<R><<<grid_for(ho.size() / 8 + 1), kThreads, sizeof(double) * 2 * ns>>>(
        F, ho, pg, max_r2, min_r2, nreal, normfft, iround, ns, proj, sums);
    RC_CUDA(cudaGetLastError());
    std::vector<double> h(2 * ns);
    RC_CUDA(cudaMemcpy(h.data(), sums, sizeof(double) * 2 * ns, cudaMemcpyDeviceToHost));
    if (power_host)
        for (int i = 0; i < ns; ++i) power_host[i] = h[ns + i] < 1. ? 0. : h[i] / h[ns + i];
    return 0;
}

template <class R>
int fsc_impl(ReconWork *w, const double *m1, const double *m2, int ori, int dim, double *fsc_host) {
    typedef typename Cx<R>::T C2;
    const Half h = make_half(ori, dim);
    RC_CUDA(w->c1.reserve(sizeof(C2) * h.size()));
    RC_CUDA(w->c2.reserve(sizeof(C2) * h.size()));
    const long long nv = (long long)h.Z * h.Y * ori;
    // maps in FP64 -> real rows of the in-place transforms
    RC_CUDA(w->vol.reserve(sizeof(double) * nv));
    for (int which = 0; which < 2; ++which) {
        RC_CUDA(cudaMemcpy(w->vol.p, which ? m2 : m1, sizeof(double) * nv, cudaMemcpyHostToDevice));
        R *dst = which ? w->c2.as<R>() : w->c1.as<R>();
        // padding to the map's own size: a plain copy into the padded rows
        k_pad_map<R><<<grid_for((long long)h.Z * h.Y * h.rowp()), kThreads>>>(w->vol.as<double>(), ori, dim, ori,
                                                                               h.rowp(), nullptr, dst);
        RC_CUDA(cudaGetLastError());
        const int st = exec_fwd<R>(w, ori, dim, dst);
        if (st) return st;
    }
    RC_CUDA(w->small.reserve(sizeof(double) * 3 * h.X));
    double *sums = w->small.as<double>();
    RC_CUDA(cudaMemset(sums, 0, sizeof(double) * 3 * h.X));
    int tst = 0;
    const int *iround1 = shell_table(w, 1, 3 * (ori / 2) * (ori / 2) + 1, 0, tst);
    if (!iround1) return tst;
    k_fsc<R><<<grid_for(h.size()), kThreads, sizeof(double) * 3 * h.X>>>(w->c1.as<C2>(), w->c2.as<C2>(), h,
                                                                          (double)h.Z * h.Y * h.N, iround1, sums);
    RC_CUDA(cudaGetLastError());
    std::vector<double> s(3 * h.X);
    RC_CUDA(cudaMemcpy(s.data(), sums, sizeof(double) * 3 * h.X, cudaMemcpyDeviceToHost));
    for (int i = 0; i < h.X; ++i) fsc_host[i] = s[i] / std::sqrt(s[h.X + i] * s[2 * h.X + i]);
    return 0;
}

}  // namespace

int recon_reconstruct(ReconWork *w, const double2 *data, const double *weight, const VolGeom &g, int ori,
                      const ReconParams &p, const double *tau2_host, double *vol_host) {
    return w->fp32 ? reconstruct_impl<float>(w, data, weight, g, ori, p, tau2_host, vol_host)
                   : reconstruct_impl<double>(w, data, weight, g, ori, p, tau2_host, vol_host);
}

int recon_projector_from_map(ReconWork *w, const double *vol_host, int ori, int dim, int pad, const VolGeom &pg,
                             int do_gridding, int min_ires, float2 *proj, double *power_host) {
    return w->fp32 ? projector_impl<float>(w, vol_host, ori, dim, pad, pg, do_gridding, min_ires, proj, power_host)
                   : projector_impl<double>(w, vol_host, ori, dim, pad, pg, do_gridding, min_ires, proj, power_host);
}

int recon_fsc(ReconWork *w, const double *m1, const double *m2, int ori, int dim, double *fsc_host) {
    return w->fp32 ? fsc_impl<float>(w, m1, m2, ori, dim, fsc_host) : fsc_impl<double>(w, m1, m2, ori, dim, fsc_host);
}

}  // namespace gbr
