/*
 * oracle_mstep.cpp -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * Double-precision restatement of the reference's reconstruction side of an
 * iteration, which the tests compare relion_gb300/csrc/k_recon.cu with:
 *   BackProjector::enforceHermitianSymmetry   src/backprojector.cpp:2148-2165
 *   BackProjector::updateSSNRarrays           src/backprojector.cpp:1041-1204
 *   BackProjector::reconstruct                src/backprojector.cpp:1379-1872
 *     (with convoluteBlobRealSpace :2483-2528, windowToOridimRealSpace
 *      :2530-2670, softMaskOutsideMap src/mask.cpp:43-96,
 *      Projector::griddingCorrect src/projector.cpp:595-628)
 *   Projector::computeFourierTransformMap     src/projector.cpp:116-593 (CPU branch)
 *   getFSC                                    src/fftw.cpp:481-525
 * C1 only (no helical or point-group symmetry), trilinear interpolator, no
 * Fourier mask, 2D images (data_dim 2).  FFTs follow FourierTransformer's
 * conventions (src/fftw.cpp:333-373): forward divided by the number of real
 * elements, inverse unscaled, FFTW half layout [Z][Y][N/2+1].
 */
#include "relion_oracle.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

namespace {

typedef std::complex<double> cd;
const double kPI = 3.14159265358979323846;  // src/macros.h:104

inline int r_round(double x) { return (x > 0) ? (int)(x + 0.5) : (int)(x - 0.5); }            // src/macros.h:197
inline int r_floor(double x) { return (x == (int)x) ? (int)x : ((x > 0) ? (int)x : (int)(x - 1)); }  // :226

// Iterative radix-2 transform, sign -1 forward / +1 inverse, unscaled.
void fft_pow2(std::vector<cd> &a, int sign) {
    const size_t n = a.size();
    for (size_t i = 1, j = 0; i < n; ++i) {
        size_t bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(a[i], a[j]);
    }
    for (size_t len = 2; len <= n; len <<= 1) {
        const double ang = 2 * kPI / (double)len * sign;
        for (size_t i = 0; i < n; i += len)
            for (size_t k = 0; k < len / 2; ++k) {
                const cd w(std::cos(ang * k), std::sin(ang * k));
                const cd u = a[i + k], v = a[i + k + len / 2] * w;
                a[i + k] = u + v;
                a[i + k + len / 2] = u - v;
            }
    }
}

// DFT of any length: radix-2 for powers of two, otherwise Bluestein's
// chirp-z algorithm (L. Bluestein, 1970: 2jk = j^2 + k^2 - (k-j)^2 turns the
// DFT into a convolution with the chirp exp(i pi m^2 / n), evaluated with
// power-of-two transforms).  The chirp phase uses m^2 mod 2n in integers.
void fft_any(std::vector<cd> &a, int sign) {
    const size_t n = a.size();
    if (n <= 1) return;
    if ((n & (n - 1)) == 0) {
        fft_pow2(a, sign);
        return;
    }
    size_t M = 1;
    while (M < 2 * n - 1) M <<= 1;
    std::vector<cd> w(n), A(M, cd(0, 0)), B(M, cd(0, 0));
    for (size_t k = 0; k < n; ++k) {
        const unsigned long long m2 = ((unsigned long long)k * k) % (2ull * n);
        const double ph = sign * kPI * (double)m2 / (double)n;
        w[k] = cd(std::cos(ph), std::sin(ph));
    }
    for (size_t k = 0; k < n; ++k) {
        A[k] = a[k] * w[k];
        B[k] = std::conj(w[k]);
        if (k) B[M - k] = std::conj(w[k]);
    }
    fft_pow2(A, -1);
    fft_pow2(B, -1);
    for (size_t k = 0; k < M; ++k) A[k] *= B[k];
    fft_pow2(A, +1);
    for (size_t k = 0; k < n; ++k) a[k] = w[k] * A[k] / (double)M;
}

// FFTW half layout of an N^dim real array: [Z][N][N/2+1], Z = N (3D) or 1 (2D).
struct Grid {
    long N, Z, Y, X;
    int dim;
    Grid(long n, int d) : N(n), Z(d == 3 ? n : 1), Y(n), X(n / 2 + 1), dim(d) {}
    size_t half() const { return (size_t)Z * Y * X; }
    size_t real() const { return (size_t)Z * Y * N; }
    // FOR_ALL_ELEMENTS_IN_FFTW_TRANSFORM (src/fftw.h:99-102)
    long kp(long k) const { return (k < X) ? k : k - Z; }
    long ip(long i) const { return (i < X) ? i : i - Y; }
};

// unscaled forward real-to-half transform
std::vector<cd> r2c(const std::vector<double> &in, const Grid &g) {
    std::vector<cd> out(g.half());
    std::vector<cd> line(g.N);
    for (long z = 0; z < g.Z; ++z)
        for (long y = 0; y < g.Y; ++y) {
            for (long x = 0; x < g.N; ++x) line[x] = cd(in[((size_t)z * g.Y + y) * g.N + x], 0.);
            fft_any(line, -1);
            for (long x = 0; x < g.X; ++x) out[((size_t)z * g.Y + y) * g.X + x] = line[x];
        }
    for (long z = 0; z < g.Z; ++z)
        for (long x = 0; x < g.X; ++x) {
            for (long y = 0; y < g.Y; ++y) line[y] = out[((size_t)z * g.Y + y) * g.X + x];
            fft_any(line, -1);
            for (long y = 0; y < g.Y; ++y) out[((size_t)z * g.Y + y) * g.X + x] = line[y];
        }
    if (g.dim == 3)
        for (long y = 0; y < g.Y; ++y)
            for (long x = 0; x < g.X; ++x) {
                for (long z = 0; z < g.Z; ++z) line[z] = out[((size_t)z * g.Y + y) * g.X + x];
                fft_any(line, -1);
                for (long z = 0; z < g.Z; ++z) out[((size_t)z * g.Y + y) * g.X + x] = line[z];
            }
    return out;
}

// unscaled inverse half-to-real transform of a Hermitian-consistent array
std::vector<double> c2r(std::vector<cd> h, const Grid &g) {
    std::vector<cd> line(g.N);
    if (g.dim == 3)
        for (long y = 0; y < g.Y; ++y)
            for (long x = 0; x < g.X; ++x) {
                for (long z = 0; z < g.Z; ++z) line[z] = h[((size_t)z * g.Y + y) * g.X + x];
                fft_any(line, +1);
                for (long z = 0; z < g.Z; ++z) h[((size_t)z * g.Y + y) * g.X + x] = line[z];
            }
    for (long z = 0; z < g.Z; ++z)
        for (long x = 0; x < g.X; ++x) {
            for (long y = 0; y < g.Y; ++y) line[y] = h[((size_t)z * g.Y + y) * g.X + x];
            fft_any(line, +1);
            for (long y = 0; y < g.Y; ++y) h[((size_t)z * g.Y + y) * g.X + x] = line[y];
        }
    std::vector<double> out(g.real());
    for (long z = 0; z < g.Z; ++z)
        for (long y = 0; y < g.Y; ++y) {
            const cd *row = &h[((size_t)z * g.Y + y) * g.X];
            for (long x = 0; x < g.N; ++x) line[x] = (x < g.X) ? row[x] : std::conj(row[g.N - x]);
            fft_any(line, +1);
            for (long x = 0; x < g.N; ++x) out[((size_t)z * g.Y + y) * g.N + x] = line[x].real();
        }
    return out;
}

inline double cabs(const cd &z) { return std::sqrt(z.real() * z.real() + z.imag() * z.imag()); }

// Backprojector / projector array: logical (k, i, j), x from 0 (src/projector.cpp:59-89)
struct Centered {
    long xdim, ydim, zdim, yinit, zinit;
    size_t at(long k, long i, long j) const { return ((size_t)(k - zinit) * ydim + (i - yinit)) * xdim + j; }
};

Centered bp_layout(const oracle_bp_geom *g) {
    return Centered{(long)g->xdim, (long)g->ydim, (long)g->zdim, (long)g->yinit, (long)g->zinit};
}

// Projector::griddingCorrect (trilinear: divide by sinc^2), logical origin at the centre
void gridding_correct(std::vector<double> &v, long ori, int dim, double pad) {
    const long h = ori / 2, Z = dim == 3 ? ori : 1;
    for (long z = 0; z < Z; ++z)
        for (long y = 0; y < ori; ++y)
            for (long x = 0; x < ori; ++x) {
                const long k = dim == 3 ? z - h : 0, i = y - h, j = x - h;
                const double r = std::sqrt((double)(k * k + i * i + j * j));
                if (r > 0.) {
                    const double rval = r / (ori * pad);
                    const double sinc = std::sin(kPI * rval) / (kPI * rval);
                    v[((size_t)z * ori + y) * ori + x] /= sinc * sinc;
                }
            }
}

// softMaskOutsideMap with the default radius (XSIZE/2) and cosine width 3
void soft_mask_outside(std::vector<double> &v, long ori, int dim) {
    const long h = ori / 2, Z = dim == 3 ? ori : 1;
    const double radius = (double)ori / 2., width = 3., radius_p = radius + width;
    double sum_bg = 0., sum = 0.;
    for (int pass = 0; pass < 2; ++pass) {
        if (pass == 1) sum_bg /= sum;
        for (long z = 0; z < Z; ++z)
            for (long y = 0; y < ori; ++y)
                for (long x = 0; x < ori; ++x) {
                    const long k = dim == 3 ? z - h : 0, i = y - h, j = x - h;
                    const double r = std::sqrt((double)(k * k + i * i + j * j));
                    double &e = v[((size_t)z * ori + y) * ori + x];
                    if (r < radius) continue;
                    if (r > radius_p) {
                        if (pass == 0) {
                            sum += 1.;
                            sum_bg += e;
                        } else {
                            e = sum_bg;
                        }
                    } else {
                        const double rc = 0.5 + 0.5 * std::cos(kPI * (radius_p - r) / width);
                        if (pass == 0) {
                            sum += rc;
                            sum_bg += rc * e;
                        } else {
                            e = (1 - rc) * e + rc * sum_bg;
                        }
                    }
                }
    }
}

// I_{3/2} and J_{3/2} in closed form (spherical Bessel functions)
double bessi1_5(double x) { return (x == 0) ? 0 : std::sqrt(2 / (kPI * x)) * (std::cosh(x) - std::sinh(x) / x); }
double bessj1_5(double x) { return (x == 0) ? 0 : std::sqrt(2 / (kPI * x)) * (std::sin(x) / x - std::cos(x)); }

// TabFtBlob (src/tabfuncs.cpp:95-121) of the order-0 Kaiser-Bessel blob
// (kaiser_Fourier_value, src/funcs.cpp:232-255) without its constant factors,
// which cancel in tab(r) / tab(0).
struct FtBlob {
    std::vector<double> t;
    double sampling;
    FtBlob(double a, double alpha, int n) : t(n), sampling(0.5 / n) {
        for (int i = 0; i < n; ++i) {
            const double w = i * sampling, s2 = 2. * kPI * a * w;
            const double sigma = std::sqrt(std::fabs(alpha * alpha - s2 * s2));
            t[i] = (s2 > alpha ? bessj1_5(sigma) : bessi1_5(sigma)) / std::pow(sigma, 1.5);
        }
    }
    double operator()(double v) const {
        const int idx = (int)(std::fabs(v) / sampling);
        return idx >= (int)t.size() ? 0. : t[idx];
    }
};

}  // namespace

extern "C" {

int oracle_bp_symmetrise(const oracle_bp_geom *g, double *data, double *weight) {
    const Centered L = bp_layout(g);
    cd *D = reinterpret_cast<cd *>(data);
    const long zfin = L.zinit + L.zdim - 1, yfin = L.yinit + L.ydim - 1;
    for (long iz = L.zinit; iz <= zfin; ++iz) {
        const long starty = (iz < 0) ? 0 : 1;
        for (long iy = starty; iy <= yfin; ++iy) {
            const size_t a = L.at(iz, iy, 0), b = L.at(-iz, -iy, 0);
            const cd fsum = D[a] + std::conj(D[b]);
            D[a] = fsum;
            D[b] = std::conj(fsum);
            const double s = weight[a] + weight[b];
            weight[a] = s;
            weight[b] = s;
        }
    }
    return 0;
}

int oracle_update_ssnr(const oracle_bp_geom *g, const double *weight, double tau2_fudge, double *tau2_io,
                       double *sigma2_out, double *dvp_out, double *cov_out, const double *fsc,
                       int64_t update_tau2_with_fsc, int64_t is_whole_instead_of_half) {
    const Centered L = bp_layout(g);
    const long ns = g->ori_size / 2 + 1;
    const double pad = (double)g->pad;
    const int max_r2 = r_round(g->r_max * pad) * r_round(g->r_max * pad);
    const double ovc = g->ref_dim == 3 ? pad * pad * pad : pad * pad;
    std::vector<double> sigma2(ns, 0.), counter(ns, 0.), tau2(tau2_io, tau2_io + ns), dvp(ns, 0.), cov(ns, 0.);
    for (long k = L.zinit; k < L.zinit + L.zdim; ++k)
        for (long i = L.yinit; i < L.yinit + L.ydim; ++i)
            for (long j = 0; j < L.xdim; ++j) {
                const int r2 = (int)(k * k + i * i + j * j);
                if (r2 < max_r2) {
                    const int ires = r_round(std::sqrt((double)r2) / pad);
                    sigma2[ires] += ovc * weight[L.at(k, i, j)];
                    counter[ires] += 1.;
                }
            }
    for (long i = 0; i < ns; ++i) {
        if (sigma2[i] > 1e-20) sigma2[i] = counter[i] / sigma2[i];
        else if (sigma2[i] == 0) sigma2[i] = 0.;
        else return -1;  // "unexpectedly small, yet non-zero sigma2 value"
    }
    std::fill(counter.begin(), counter.end(), 0.);
    if (update_tau2_with_fsc) {
        for (long i = 0; i < ns; ++i) {
            double myfsc = std::max(0.001, fsc[i]);
            if (is_whole_instead_of_half) myfsc = std::sqrt(2. * myfsc / (myfsc + 1.));
            myfsc = std::min(0.999, myfsc);
            double myssnr = myfsc / (1. - myfsc);
            myssnr *= tau2_fudge;
            tau2[i] = myssnr * sigma2[i];
            dvp[i] = myssnr;
        }
    }
    for (long k = L.zinit; k < L.zinit + L.zdim; ++k)
        for (long i = L.yinit; i < L.yinit + L.ydim; ++i)
            for (long j = 0; j < L.xdim; ++j) {
                const int r2 = (int)(k * k + i * i + j * j);
                if (r2 < max_r2) {
                    const int ires = r_round(std::sqrt((double)r2) / pad);
                    const double invw = weight[L.at(k, i, j)];
                    double invtau2;
                    if (tau2[ires] > 0.) invtau2 = 1. / (ovc * tau2_fudge * tau2[ires]);
                    else if (tau2[ires] == 0.) invtau2 = 1. / (0.001 * invw);
                    else return -2;  // negative tau2
                    if (!update_tau2_with_fsc) dvp[ires] += invw / invtau2;
                    if (invw / invtau2 >= 1.) cov[ires] += 1.;
                    counter[ires] += 1.;
                }
            }
    if (!update_tau2_with_fsc)
        for (long i = 0; i < ns; ++i) {
            if (i > g->r_max) dvp[i] = 0.;
            else if (counter[i] < 0.001) dvp[i] = 999.;
            else dvp[i] /= counter[i];
        }
    for (long i = 0; i < ns; ++i)
        if (counter[i] > 0.) cov[i] /= counter[i];
    std::copy(tau2.begin(), tau2.end(), tau2_io);
    std::copy(sigma2.begin(), sigma2.end(), sigma2_out);
    std::copy(dvp.begin(), dvp.end(), dvp_out);
    std::copy(cov.begin(), cov.end(), cov_out);
    return 0;
}

int oracle_reconstruct(const oracle_bp_geom *g, const double *data, const double *weight,
                       const oracle_recon_params *p, const double *tau2, double *vol_out) {
    const Centered L = bp_layout(g);
    const cd *D = reinterpret_cast<const cd *>(data);
    const int dim = (int)g->ref_dim;
    const double pad = (double)g->pad;
    const long ori = g->ori_size, r_max = g->r_max, pad_size = L.ydim;
    const int max_r2 = r_round(r_max * pad) * r_round(r_max * pad);
    const double ovc = dim == 3 ? pad * pad * pad : pad * pad;
    const Grid G(pad_size, dim);
    auto r2_of = [&](long k, long i, long j) {
        const long kp = G.kp(k), ip = G.ip(i);
        return (int)(kp * kp + ip * ip + j * j);
    };
    // Projector::decenter of the weight (src/projector.h:249-260) and the MAP term
    std::vector<double> Fweight(G.half(), 0.);
    for (long k = 0; k < G.Z; ++k)
        for (long i = 0; i < G.Y; ++i)
            for (long j = 0; j < G.X; ++j) {
                const long kp = G.kp(k), ip = G.ip(i);
                const int r2 = r2_of(k, i, j);
                const size_t o = ((size_t)k * G.Y + i) * G.X + j;
                if (r2 <= max_r2) Fweight[o] = weight[L.at(kp, ip, j)];
                if (p->do_map && r2 < max_r2) {
                    const int ires = r_round(std::sqrt((double)r2) / pad);
                    const double invw = Fweight[o];
                    double invtau2;
                    if (tau2[ires] > 0.) invtau2 = 1. / (ovc * p->tau2_fudge * tau2[ires]);
                    else invtau2 = (invw > 1e-20) ? 1. / (0.001 * invw) : 0.;
                    if (ires >= p->minres_map) Fweight[o] = invw + invtau2;
                }
            }
    std::vector<cd> Fconv(G.half(), cd(0, 0));
    if (p->skip_gridding || p->max_iter_preweight <= 0) {
        for (long k = 0; k < G.Z; ++k)
            for (long i = 0; i < G.Y; ++i)
                for (long j = 0; j < G.X; ++j)
                    if (r2_of(k, i, j) <= max_r2) Fconv[((size_t)k * G.Y + i) * G.X + j] = D[L.at(G.kp(k), G.ip(i), j)];
        std::vector<double> radavg(r_max, 0.), counter(r_max, 0.);
        const int round_max_r2 = r_round(r_max * pad * r_max * pad);
        for (long k = 0; k < G.Z; ++k)
            for (long i = 0; i < G.Y; ++i)
                for (long j = 0; j < G.X; ++j) {
                    const int r2 = r2_of(k, i, j);
                    if (r2 < round_max_r2) {
                        const int ires = r_floor(std::sqrt((double)r2) / pad);
                        if (ires >= r_max) return -3;
                        radavg[ires] += Fweight[((size_t)k * G.Y + i) * G.X + j];
                        counter[ires] += 1.;
                    }
                }
        for (long i = 0; i < r_max; ++i) {
            if (counter[i] > 0. || radavg[i] > 0.) radavg[i] /= 1000. * counter[i];
            else return -4;  // "zeros in counter or radavg_weight"
        }
        for (long k = 0; k < G.Z; ++k)
            for (long i = 0; i < G.Y; ++i)
                for (long j = 0; j < G.X; ++j) {
                    const int r2 = r2_of(k, i, j);
                    const int ires = r_floor(std::sqrt((double)r2) / pad);
                    const size_t o = ((size_t)k * G.Y + i) * G.X + j;
                    const double w = std::max(Fweight[o], radavg[(ires < r_max) ? ires : (r_max - 1)]);
                    if (w != 0.) Fconv[o] /= w;
                }
    } else {
        for (double &w : Fweight) w /= p->normalise;
        std::vector<double> Fnew(G.half(), 0.);
        for (long k = 0; k < G.Z; ++k)
            for (long i = 0; i < G.Y; ++i)
                for (long j = 0; j < G.X; ++j)
                    if (r2_of(k, i, j) < max_r2) Fnew[((size_t)k * G.Y + i) * G.X + j] = 1.;
        const FtBlob blob(1.9 * 2., 15., 10000);
        const double norm_blob = blob(0.);
        const long padh = pad_size / 2;
        const double nreal = (double)G.real();
        for (int it = 0; it < p->max_iter_preweight; ++it) {
            for (size_t n = 0; n < G.half(); ++n) Fconv[n] = cd(Fnew[n] * Fweight[n], 0.);
            // convoluteBlobRealSpace(transformer, false)
            std::vector<double> M = c2r(Fconv, G);
            for (long k = 0; k < G.Z; ++k)
                for (long i = 0; i < G.Y; ++i)
                    for (long j = 0; j < G.N; ++j) {
                        const long kp = (k < padh) ? k : k - pad_size, ip = (i < padh) ? i : i - pad_size,
                                   jp = (j < padh) ? j : j - pad_size;
                        const long kk = dim == 3 ? kp : 0;
                        const double rval = std::sqrt((double)(kk * kk + ip * ip + jp * jp)) / (ori * pad);
                        M[((size_t)k * G.Y + i) * G.N + j] *= blob(rval) / norm_blob;
                    }
            Fconv = r2c(M, G);
            for (cd &z : Fconv) z /= nreal;
            for (long k = 0; k < G.Z; ++k)
                for (long i = 0; i < G.Y; ++i)
                    for (long j = 0; j < G.X; ++j)
                        if (r2_of(k, i, j) < max_r2) {
                            const size_t o = ((size_t)k * G.Y + i) * G.X + j;
                            Fnew[o] /= std::max(1e-6, cabs(Fconv[o]));
                        }
        }
        std::fill(Fconv.begin(), Fconv.end(), cd(0, 0));
        for (long k = 0; k < G.Z; ++k)
            for (long i = 0; i < G.Y; ++i)
                for (long j = 0; j < G.X; ++j)
                    if (r2_of(k, i, j) <= max_r2) {
                        const size_t o = ((size_t)k * G.Y + i) * G.X + j;
                        Fconv[o] = D[L.at(G.kp(k), G.ip(i), j)] / p->normalise;
                    }
        for (size_t n = 0; n < G.half(); ++n) Fconv[n] *= Fnew[n];
    }
    // windowToOridimRealSpace: windowFourierTransform (src/fftw.h:809-857) to the padded box
    long No = r_round(pad * ori);
    No += No % 2;
    const Grid O(No, dim);
    std::vector<cd> Fo(O.half(), cd(0, 0));
    if (O.X > G.X) {
        const long mr2 = (G.X - 1) * (G.X - 1);
        for (long k = 0; k < G.Z; ++k)
            for (long i = 0; i < G.Y; ++i)
                for (long j = 0; j < G.X; ++j) {
                    const long kp = G.kp(k), ip = G.ip(i);
                    if (kp * kp + ip * ip + j * j <= mr2) {
                        const long ko = kp < 0 ? kp + O.Z : kp, io = ip < 0 ? ip + O.Y : ip;
                        Fo[((size_t)ko * O.Y + io) * O.X + j] = Fconv[((size_t)k * G.Y + i) * G.X + j];
                    }
                }
    } else {
        for (long k = 0; k < O.Z; ++k)
            for (long i = 0; i < O.Y; ++i)
                for (long j = 0; j < O.X; ++j) {
                    const long kp = O.kp(k), ip = O.ip(i);
                    const long ki = kp < 0 ? kp + G.Z : kp, ii = ip < 0 ? ip + G.Y : ip;
                    Fo[((size_t)k * O.Y + i) * O.X + j] = Fconv[((size_t)ki * G.Y + ii) * G.X + j];
                }
    }
    // CenterFFTbySign (src/fftw.h:389-402)
    for (long k = 0; k < O.Z; ++k)
        for (long i = 0; i < O.Y; ++i)
            for (long j = 0; j < O.X; ++j)
                if ((k ^ i ^ j) & 1) Fo[((size_t)k * O.Y + i) * O.X + j] *= -1.;
    const std::vector<double> Mo = c2r(Fo, O);
    const double normfft = dim == 3 ? pad * pad * pad * ori : pad * pad;
    const long Zv = dim == 3 ? ori : 1, off = No / 2 - ori / 2;
    std::vector<double> v((size_t)Zv * ori * ori);
    for (long z = 0; z < Zv; ++z)
        for (long y = 0; y < ori; ++y)
            for (long x = 0; x < ori; ++x) {
                const long zo = dim == 3 ? z + off : 0;
                v[((size_t)z * ori + y) * ori + x] = Mo[((size_t)zo * No + (y + off)) * No + (x + off)] / normfft;
            }
    soft_mask_outside(v, ori, dim);
    gridding_correct(v, ori, dim, pad);
    std::copy(v.begin(), v.end(), vol_out);
    return 0;
}

int oracle_projector_from_map(int64_t ori, int64_t ref_dim, int64_t padding_factor, const double *vol,
                              int64_t current_size, int64_t do_gridding, int64_t min_ires, double *proj_out,
                              double *power_out) {
    const int dim = (int)ref_dim;
    const double pad = (double)padding_factor;
    long No = r_round(pad * ori);
    No += No % 2;
    const long Zv = dim == 3 ? ori : 1, h = ori / 2;
    std::vector<double> v(vol, vol + (size_t)Zv * ori * ori);
    if (do_gridding) gridding_correct(v, ori, dim, pad);
    const Grid O(No, dim);
    std::vector<double> Mpad(O.real(), 0.);
    const long off = No / 2 - h;
    for (long z = 0; z < Zv; ++z)
        for (long y = 0; y < ori; ++y)
            for (long x = 0; x < ori; ++x) {
                const long zo = dim == 3 ? z + off : 0;
                Mpad[((size_t)zo * No + (y + off)) * No + (x + off)] = v[((size_t)z * ori + y) * ori + x];
            }
    std::vector<cd> F = r2c(Mpad, O);
    const double nreal = (double)O.real();
    for (long k = 0; k < O.Z; ++k)
        for (long i = 0; i < O.Y; ++i)
            for (long j = 0; j < O.X; ++j) {
                cd &z = F[((size_t)k * O.Y + i) * O.X + j];
                z /= nreal;
                if ((k ^ i ^ j) & 1) z *= -1.;
            }
    // Projector::initZeros(current_size)
    long r_max = current_size < 0 ? ori / 2 : current_size / 2;
    r_max = std::min<long>(r_max, ori / 2);
    const long pad_size = 2 * (r_round(pad * r_max) + 1) + 1;
    const Centered L{pad_size / 2 + 1, pad_size, dim == 3 ? pad_size : 1, -(pad_size / 2),
                     dim == 3 ? -(pad_size / 2) : 0};
    cd *P = reinterpret_cast<cd *>(proj_out);
    std::fill(P, P + (size_t)L.xdim * L.ydim * L.zdim, cd(0, 0));
    const long ns = ori / 2 + 1;
    std::vector<double> ps(ns, 0.), counter(ns, 0.);
    const int max_r2 = r_round(r_max * pad) * r_round(r_max * pad);
    const int min_r2 = min_ires > 0 ? r_round(min_ires * pad) * r_round(min_ires * pad) : -1;
    const double normfft = dim == 3 ? pad * pad * pad * ori : pad * pad;
    for (long k = 0; k < O.Z; ++k)
        for (long i = 0; i < O.Y; ++i)
            for (long j = 0; j < O.X; ++j) {
                const long kp = O.kp(k), ip = O.ip(i);
                const int r2 = (int)(kp * kp + ip * ip + j * j);
                if (r2 <= max_r2) {
                    cd &e = P[L.at(kp, ip, j)];
                    e = F[((size_t)k * O.Y + i) * O.X + j] * normfft;
                    const int ires = r_round(std::sqrt((double)r2) / pad);
                    ps[ires] += std::norm(e) / 2.;
                    counter[ires] += 1.;
                    if (r2 <= min_r2) e = cd(0, 0);
                }
            }
    if (power_out)
        for (long i = 0; i < ns; ++i) power_out[i] = counter[i] < 1. ? 0. : ps[i] / counter[i];
    return 0;
}

int oracle_fsc(int64_t ori, int64_t ref_dim, const double *m1, const double *m2, double *fsc) {
    const Grid G(ori, (int)ref_dim);
    std::vector<double> a(m1, m1 + G.real()), b(m2, m2 + G.real());
    std::vector<cd> F1 = r2c(a, G), F2 = r2c(b, G);
    const double nreal = (double)G.real();
    std::vector<double> num(G.X, 0.), d1(G.X, 0.), d2(G.X, 0.);
    for (long k = 0; k < G.Z; ++k)
        for (long i = 0; i < G.Y; ++i)
            for (long j = 0; j < G.X; ++j) {
                const long kp = G.kp(k), ip = G.ip(i);
                const int idx = r_round(std::sqrt((double)(kp * kp + ip * ip + j * j)));
                if (idx >= G.X) continue;
                const size_t o = ((size_t)k * G.Y + i) * G.X + j;
                const cd z1 = F1[o] / nreal, z2 = F2[o] / nreal;
                num[idx] += z1.real() * z2.real() + z1.imag() * z2.imag();
                const double a1 = cabs(z1), a2 = cabs(z2);
                d1[idx] += a1 * a1;
                d2[idx] += a2 * a2;
            }
    for (long i = 0; i < G.X; ++i) fsc[i] = num[i] / std::sqrt(d1[i] * d2[i]);
    return 0;
}

}  // extern "C"
