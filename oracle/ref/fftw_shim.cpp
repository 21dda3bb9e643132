// fftw_shim.cpp -- TEST INFRASTRUCTURE ONLY: the FFTW3 calls the
// reference's src/fftw.cpp makes (oracle/ref/shim/fftw3.h), implemented on a
// double-precision FFT written for this project, so that the reference's CPU
// sources can be linked into oracle/_ref/ref_pin without FFTW.
//
// Transforms follow FFTW's definitions: unnormalised, exponent sign -1 for
// the forward and +1 for the backward transform, row-major arrays, the last
// dimension halved (n/2 + 1) on the complex side of real transforms; the
// complex-to-real transform reads only the stored half (the imaginary parts
// of the self-conjugate elements do not enter the real output).
// One-dimensional transforms: iterative radix-2 for powers of two, otherwise
// Bluestein's chirp-z algorithm (L. Bluestein, 1970), which rewrites a DFT of
// any length as a convolution evaluated with power-of-two transforms.
#include "fftw3.h"

#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <vector>

typedef std::complex<double> cd;

struct gbr_shim_plan_s {
    int kind;       // 0 r2c, 1 c2r, 2 c2c
    int rank;
    int n[3];
    int sign;       // c2c only
};

namespace {

const double kPi = 3.14159265358979323846;

bool is_pow2(size_t n) { return n && !(n & (n - 1)); }

void fft_pow2(std::vector<cd> &a, int sign) {
    const size_t n = a.size();
    for (size_t i = 1, j = 0; i < n; ++i) {
        size_t bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(a[i], a[j]);
    }
    for (size_t len = 2; len <= n; len <<= 1) {
        const double ang = sign * 2 * kPi / (double)len;
        for (size_t i = 0; i < n; i += len)
            for (size_t k = 0; k < len / 2; ++k) {
                const cd w(std::cos(ang * (double)k), std::sin(ang * (double)k));
                const cd u = a[i + k], v = a[i + k + len / 2] * w;
                a[i + k] = u + v;
                a[i + k + len / 2] = u - v;
            }
    }
}

// DFT of any length, exponent sign `sign`, unnormalised.
void dft(std::vector<cd> &a, int sign) {
    const size_t n = a.size();
    if (n <= 1) return;
    if (is_pow2(n)) {
        fft_pow2(a, sign);
        return;
    }
    // j k = (j^2 + k^2 - (k - j)^2) / 2
    size_t m = 1;
    while (m < 2 * n - 1) m <<= 1;
    std::vector<cd> w(n), A(m, cd(0, 0)), B(m, cd(0, 0));
    for (size_t k = 0; k < n; ++k) {
        const double ang = sign * kPi * (double)((k * k) % (2 * n)) / (double)n;
        w[k] = cd(std::cos(ang), std::sin(ang));
    }
    for (size_t k = 0; k < n; ++k) A[k] = a[k] * w[k];
    B[0] = std::conj(w[0]);
    for (size_t k = 1; k < n; ++k) B[k] = B[m - k] = std::conj(w[k]);
    fft_pow2(A, -1);
    fft_pow2(B, -1);
    for (size_t i = 0; i < m; ++i) A[i] *= B[i];
    fft_pow2(A, +1);
    for (size_t k = 0; k < n; ++k) a[k] = A[k] * w[k] / (double)m;
}

// Complex transform along axis `ax` of a row-major array of dims d[0..rank-1].
void along_axis(std::vector<cd> &v, const int *d, int rank, int ax, int sign) {
    size_t inner = 1, outer = 1;
    for (int k = ax + 1; k < rank; ++k) inner *= (size_t)d[k];
    for (int k = 0; k < ax; ++k) outer *= (size_t)d[k];
    const size_t len = (size_t)d[ax];
    std::vector<cd> line(len);
    for (size_t o = 0; o < outer; ++o)
        for (size_t i = 0; i < inner; ++i) {
            const size_t base = o * len * inner + i;
            for (size_t k = 0; k < len; ++k) line[k] = v[base + k * inner];
            dft(line, sign);
            for (size_t k = 0; k < len; ++k) v[base + k * inner] = line[k];
        }
}

gbr_shim_plan_s *make(int kind, int rank, const int *n, int sign) {
    if (rank < 1 || rank > 3) return nullptr;
    gbr_shim_plan_s *p = new gbr_shim_plan_s();
    p->kind = kind;
    p->rank = rank;
    for (int k = 0; k < rank; ++k) p->n[k] = n[k];
    p->sign = sign;
    return p;
}

template <class R>
void r2c(const gbr_shim_plan_s *p, const R *in, R *out2) {
    const int rank = p->rank;
    const int last = p->n[rank - 1], half = last / 2 + 1;
    size_t rows = 1;
    for (int k = 0; k < rank - 1; ++k) rows *= (size_t)p->n[k];
    // last axis: real -> half complex; then the other axes, complex
    std::vector<cd> v(rows * half);
    std::vector<cd> line(last);
    for (size_t r = 0; r < rows; ++r) {
        for (int x = 0; x < last; ++x) line[x] = cd((double)in[r * last + x], 0.0);
        dft(line, -1);
        for (int x = 0; x < half; ++x) v[r * half + x] = line[x];
    }
    int d[3];
    for (int k = 0; k < rank; ++k) d[k] = p->n[k];
    d[rank - 1] = half;
    for (int ax = 0; ax < rank - 1; ++ax) along_axis(v, d, rank, ax, -1);
    for (size_t i = 0; i < v.size(); ++i) {
        out2[2 * i] = (R)v[i].real();
        out2[2 * i + 1] = (R)v[i].imag();
    }
}

template <class R>
void c2r(const gbr_shim_plan_s *p, const R *in2, R *out) {
    const int rank = p->rank;
    const int last = p->n[rank - 1], half = last / 2 + 1;
    size_t rows = 1;
    for (int k = 0; k < rank - 1; ++k) rows *= (size_t)p->n[k];
    std::vector<cd> v(rows * half);
    for (size_t i = 0; i < v.size(); ++i) v[i] = cd((double)in2[2 * i], (double)in2[2 * i + 1]);
    int d[3];
    for (int k = 0; k < rank; ++k) d[k] = p->n[k];
    d[rank - 1] = half;
    for (int ax = 0; ax < rank - 1; ++ax) along_axis(v, d, rank, ax, +1);
    // last axis: half complex -> real; element x of the full line is the
    // stored one for x <= last/2 and the conjugate of (last - x) otherwise;
    // the self-conjugate elements count with their real part only
    std::vector<cd> line(last);
    for (size_t r = 0; r < rows; ++r) {
        for (int x = 0; x < last; ++x) {
            if (x < half) {
                line[x] = v[r * half + x];
                if (x == 0 || 2 * x == last) line[x] = cd(line[x].real(), 0.0);
            } else {
                line[x] = std::conj(v[r * half + (last - x)]);
            }
        }
        dft(line, +1);
        for (int x = 0; x < last; ++x) out[r * last + x] = (R)line[x].real();
    }
}

template <class R>
void c2c(const gbr_shim_plan_s *p, const R *in2, R *out2) {
    size_t total = 1;
    for (int k = 0; k < p->rank; ++k) total *= (size_t)p->n[k];
    std::vector<cd> v(total);
    for (size_t i = 0; i < total; ++i) v[i] = cd((double)in2[2 * i], (double)in2[2 * i + 1]);
    for (int ax = 0; ax < p->rank; ++ax) along_axis(v, p->n, p->rank, ax, p->sign);
    for (size_t i = 0; i < total; ++i) {
        out2[2 * i] = (R)v[i].real();
        out2[2 * i + 1] = (R)v[i].imag();
    }
}

}  // namespace

extern "C" {

fftw_plan fftw_plan_dft_r2c(int rank, const int *n, double *, fftw_complex *, unsigned) { return make(0, rank, n, -1); }
fftw_plan fftw_plan_dft_c2r(int rank, const int *n, fftw_complex *, double *, unsigned) { return make(1, rank, n, +1); }
fftw_plan fftw_plan_dft(int rank, const int *n, fftw_complex *, fftw_complex *, int sign, unsigned) {
    return make(2, rank, n, sign);
}
void fftw_execute_dft_r2c(const fftw_plan p, double *in, fftw_complex *out) { r2c(p, in, &out[0][0]); }
void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex *in, double *out) { c2r(p, &in[0][0], out); }
void fftw_execute_dft(const fftw_plan p, fftw_complex *in, fftw_complex *out) { c2c(p, &in[0][0], &out[0][0]); }
void fftw_execute(const fftw_plan) { std::abort(); }  // plans are executed on explicit arrays only
void fftw_destroy_plan(fftw_plan p) { delete p; }
void fftw_cleanup(void) {}
void *fftw_malloc(size_t n) { return std::malloc(n); }
void fftw_free(void *p) { std::free(p); }
void fftw_plan_with_nthreads(int) {}
int fftw_init_threads(void) { return 1; }
void fftw_cleanup_threads(void) {}

fftwf_plan fftwf_plan_dft_r2c(int rank, const int *n, float *, fftwf_complex *, unsigned) {
    return make(0, rank, n, -1);
}
fftwf_plan fftwf_plan_dft_c2r(int rank, const int *n, fftwf_complex *, float *, unsigned) {
    return make(1, rank, n, +1);
}
fftwf_plan fftwf_plan_dft(int rank, const int *n, fftwf_complex *, fftwf_complex *, int sign, unsigned) {
    return make(2, rank, n, sign);
}
void fftwf_execute_dft_r2c(const fftwf_plan p, float *in, fftwf_complex *out) { r2c(p, in, &out[0][0]); }
void fftwf_execute_dft_c2r(const fftwf_plan p, fftwf_complex *in, float *out) { c2r(p, &in[0][0], out); }
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex *in, fftwf_complex *out) { c2c(p, &in[0][0], &out[0][0]); }
void fftwf_execute(const fftwf_plan) { std::abort(); }
void fftwf_destroy_plan(fftwf_plan p) { delete p; }
void fftwf_cleanup(void) {}
void *fftwf_malloc(size_t n) { return std::malloc(n); }
void fftwf_free(void *p) { std::free(p); }
void fftwf_plan_with_nthreads(int) {}
int fftwf_init_threads(void) { return 1; }
void fftwf_cleanup_threads(void) {}

}  // extern "C"
