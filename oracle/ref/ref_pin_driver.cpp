// ref_pin_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A command-line driver that runs the reference's own CPU code for the
// building blocks of the E-step and the reconstruction side, so that the
// oracle's restatements can be checked against the reference itself.  It is
// compiled by oracle/build_ref.sh together with the reference's sources
// (where they lie, unmodified) and the shims of oracle/ref/shim; it is never
// part of the product and nothing under relion_gb300/ loads it.
//
//   ref_pin <mode> <request file> <response file>
//
// Request and response are flat arrays of float64 (native byte order); the
// layout of each mode is given below.  Reference functions called:
//   project      Projector::project            (src/projector.cpp:630)
//   backproject  BackProjector::backproject2Dto3D (src/backprojector.cpp:55)
//   ctf          CTF::setValues / initialise / getFftwImage (src/ctf.cpp:211, :314)
//   sampling     HealpixSampling::initialise, getOrientations,
//                getTranslationsInPixel      (src/healpix_sampling.cpp)
//   shift        shiftImageInFourierTransform (src/fftw.cpp)
//   euler        Euler_angles2matrix          (src/euler.cpp)
//   reconstruct  BackProjector::reconstruct   (src/backprojector.cpp:1379)
//   fouriermap   Projector::computeFourierTransformMap (src/projector.cpp:116)
#include "src/backprojector.h"
#include "src/ctf.h"
#include "src/euler.h"
#include "src/fftw.h"
#include "src/healpix_sampling.h"
#include "src/projector.h"

#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

// The version string the reference's build generates from src/macros.cpp.in.
const char *g_RELION_VERSION = "reference sources (oracle build)";

namespace {

std::vector<double> read_all(const char *path) {
    FILE *f = std::fopen(path, "rb");
    if (!f) throw std::runtime_error(std::string("cannot open ") + path);
    std::vector<double> v;
    double buf[4096];
    size_t n;
    while ((n = std::fread(buf, sizeof(double), 4096, f)) > 0) v.insert(v.end(), buf, buf + n);
    std::fclose(f);
    return v;
}

void write_all(const char *path, const std::vector<double> &v) {
    FILE *f = std::fopen(path, "wb");
    if (!f) throw std::runtime_error(std::string("cannot write ") + path);
    if (!v.empty() && std::fwrite(v.data(), sizeof(double), v.size(), f) != v.size())
        throw std::runtime_error("short write");
    std::fclose(f);
}

struct Reader {
    const std::vector<double> &v;
    size_t i = 0;
    double d() {
        if (i >= v.size()) throw std::runtime_error("request too short");
        return v[i++];
    }
    long l() { return (long)d(); }
};

Matrix2D<RFLOAT> read_matrix(Reader &r) {
    Matrix2D<RFLOAT> A(3, 3);
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) A(a, b) = r.d();
    return A;
}

// A padded half volume [zdim][ydim][xdim] with origin (0, yinit, zinit).
void read_volume(Reader &r, MultidimArray<Complex> &data, long xdim, long ydim, long zdim, long yinit, long zinit) {
    data.resize(zdim, ydim, xdim);
    data.yinit = yinit;
    data.zinit = zinit;
    data.xinit = 0;
    for (long n = 0; n < zdim * ydim * xdim; ++n) {
        const double re = r.d(), im = r.d();
        data.data[n] = Complex(re, im);
    }
}

// project: ori, pad, r_max, xdim, ydim, zdim, yinit, zinit, data (complex),
//          size, nmat, nmat x 3x3 matrices
// response: nmat x [size][size/2+1] complex
void mode_project(Reader &r, std::vector<double> &out) {
    const long ori = r.l(), pad = r.l(), r_max = r.l();
    const long xdim = r.l(), ydim = r.l(), zdim = r.l(), yinit = r.l(), zinit = r.l();
    Projector P(ori, TRILINEAR, (float)pad, 10, 2);
    P.r_max = r_max;
    P.ref_dim = 3;
    P.pad_size = ydim;
    read_volume(r, P.data, xdim, ydim, zdim, yinit, zinit);
    const long size = r.l(), nmat = r.l();
    for (long k = 0; k < nmat; ++k) {
        Matrix2D<RFLOAT> A = read_matrix(r);
        MultidimArray<Complex> f2d(size, size / 2 + 1);
        f2d.initZeros();
        P.project(f2d, A);
        for (long n = 0; n < (long)MULTIDIM_SIZE(f2d); ++n) {
            out.push_back(f2d.data[n].real);
            out.push_back(f2d.data[n].imag);
        }
    }
}

// backproject: ori, pad, current_size, size, nimg, then per image a 3x3
//              matrix, [size][size/2+1] complex and [size][size/2+1] weights
// response: xdim, ydim, zdim, yinit, zinit, data (complex), weight
void mode_backproject(Reader &r, std::vector<double> &out) {
    const long ori = r.l(), pad = r.l(), cur = r.l(), size = r.l(), nimg = r.l();
    BackProjector B(ori, 3, "C1", TRILINEAR, (float)pad, 10, 0, 1.9, 15, 2, true);
    B.initZeros(cur);
    for (long k = 0; k < nimg; ++k) {
        Matrix2D<RFLOAT> A = read_matrix(r);
        MultidimArray<Complex> f2d(size, size / 2 + 1);
        MultidimArray<RFLOAT> w(size, size / 2 + 1);
        for (long n = 0; n < (long)MULTIDIM_SIZE(f2d); ++n) {
            const double re = r.d(), im = r.d();
            f2d.data[n] = Complex(re, im);
        }
        for (long n = 0; n < (long)MULTIDIM_SIZE(w); ++n) w.data[n] = r.d();
        B.backproject2Dto3D(f2d, A, &w);
    }
    out.push_back(XSIZE(B.data));
    out.push_back(YSIZE(B.data));
    out.push_back(ZSIZE(B.data));
    out.push_back(STARTINGY(B.data));
    out.push_back(STARTINGZ(B.data));
    for (long n = 0; n < (long)MULTIDIM_SIZE(B.data); ++n) {
        out.push_back(B.data.data[n].real);
        out.push_back(B.data.data[n].imag);
    }
    for (long n = 0; n < (long)MULTIDIM_SIZE(B.weight); ++n) out.push_back(B.weight.data[n]);
}

// ctf: ori, angpix, n, then per CTF defU, defV, defAng, kV, Cs, Q0, Bfac,
//      scale, phase_shift
// response: n x [ori][ori/2+1] (do_damping, no padding, not abs)
void mode_ctf(Reader &r, std::vector<double> &out) {
    const long ori = r.l();
    const double angpix = r.d();
    const long n = r.l();
    for (long k = 0; k < n; ++k) {
        const double dU = r.d(), dV = r.d(), dA = r.d(), kV = r.d(), Cs = r.d(), Q0 = r.d(), Bf = r.d(),
                     sc = r.d(), ph = r.d();
        CTF ctf;
        ctf.setValues(dU, dV, dA, kV, Cs, Q0, Bf, sc, ph);
        MultidimArray<RFLOAT> img(ori, ori / 2 + 1);
        ctf.getFftwImage(img, ori, ori, angpix, false, false, false, true, false, false);
        for (long q = 0; q < (long)MULTIDIM_SIZE(img); ++q) out.push_back(img.data[q]);
    }
}

// sampling: order, psi_step, offset_range, offset_step, pixel, oversampling
// response: ndir, npsi, ntrans, then per (idir, ipsi) the oversampled
//           (rot, tilt, psi) triplets, then per itrans the oversampled
//           (x, y) translations in pixels
void mode_sampling(Reader &r, std::vector<double> &out) {
    HealpixSampling S;
    S.healpix_order = (int)r.l();
    S.psi_step = r.d();
    S.offset_range = r.d();
    S.offset_step = r.d();
    const double pix = r.d();
    const int ov = (int)r.l();
    S.fn_sym = "C1";
    S.limit_tilt = -91.;
    S.initialise(3);
    S.random_perturbation = 0.;
    const long ndir = S.NrDirections(), npsi = S.NrPsiSamplings(), ntr = S.NrTranslationalSamplings();
    out.push_back(ndir);
    out.push_back(npsi);
    out.push_back(ntr);
    std::vector<int> pdir, ppsi;
    std::vector<RFLOAT> dprior, pprior, rot, tilt, psi, tx, ty, tz;
    for (long id = 0; id < ndir; ++id)
        for (long ip = 0; ip < npsi; ++ip) {
            S.getOrientations(id, ip, ov, rot, tilt, psi, pdir, dprior, ppsi, pprior);
            for (size_t q = 0; q < rot.size(); ++q) {
                out.push_back(rot[q]);
                out.push_back(tilt[q]);
                out.push_back(psi[q]);
            }
        }
    for (long it = 0; it < ntr; ++it) {
        S.getTranslationsInPixel(it, ov, pix, tx, ty, tz);
        for (size_t q = 0; q < tx.size(); ++q) {
            out.push_back(tx[q]);
            out.push_back(ty[q]);
        }
    }
}

// shift: size, oridim, xshift, yshift, [size][size/2+1] complex
// response: the shifted image
void mode_shift(Reader &r, std::vector<double> &out) {
    const long size = r.l();
    const double oridim = r.d(), sx = r.d(), sy = r.d();
    MultidimArray<Complex> in(size, size / 2 + 1), o;
    for (long n = 0; n < (long)MULTIDIM_SIZE(in); ++n) {
        const double re = r.d(), im = r.d();
        in.data[n] = Complex(re, im);
    }
    shiftImageInFourierTransform(in, o, oridim, sx, sy);
    for (long n = 0; n < (long)MULTIDIM_SIZE(o); ++n) {
        out.push_back(o.data[n].real);
        out.push_back(o.data[n].imag);
    }
}

// euler: n, n x (rot, tilt, psi)   response: n x 3x3
void mode_euler(Reader &r, std::vector<double> &out) {
    const long n = r.l();
    for (long k = 0; k < n; ++k) {
        const double a = r.d(), b = r.d(), g = r.d();
        Matrix2D<RFLOAT> A;
        Euler_angles2matrix(a, b, g, A, false);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) out.push_back(A(i, j));
    }
}

// reconstruct: ori, pad, current_size, skip_gridding, max_iter_preweight,
//              do_map, tau2_fudge, normalise, minres_map, xdim, ydim, zdim,
//              data (complex), weight, tau2 [ori/2+1]
// response: the real-space map [ori]^3
void mode_reconstruct(Reader &r, std::vector<double> &out) {
    const long ori = r.l(), pad = r.l(), cur = r.l();
    const bool skip = r.l() != 0;
    const int iters = (int)r.l();
    const bool do_map = r.l() != 0;
    const double fudge = r.d(), normalise = r.d();
    const int minres = (int)r.l();
    BackProjector B(ori, 3, "C1", TRILINEAR, (float)pad, 10, 0, 1.9, 15, 2, skip);
    B.initZeros(cur);
    const long xdim = r.l(), ydim = r.l(), zdim = r.l();
    if (xdim != XSIZE(B.data) || ydim != YSIZE(B.data) || zdim != ZSIZE(B.data))
        throw std::runtime_error("reconstruct: volume dimensions differ from BackProjector::initZeros");
    for (long n = 0; n < (long)MULTIDIM_SIZE(B.data); ++n) {
        const double re = r.d(), im = r.d();
        B.data.data[n] = Complex(re, im);
    }
    for (long n = 0; n < (long)MULTIDIM_SIZE(B.weight); ++n) B.weight.data[n] = r.d();
    MultidimArray<RFLOAT> tau2(ori / 2 + 1), vol;
    for (long n = 0; n < ori / 2 + 1; ++n) tau2.data[n] = r.d();
    B.reconstruct(vol, iters, do_map, tau2, fudge, normalise, minres, false, nullptr);
    for (long n = 0; n < (long)MULTIDIM_SIZE(vol); ++n) out.push_back(vol.data[n]);
}

// fouriermap: ori, pad, current_size, do_gridding, min_ires, map [ori]^3
// response: xdim, ydim, zdim, yinit, zinit, r_max, data (complex),
//           power_spectrum [ori/2+1]
void mode_fouriermap(Reader &r, std::vector<double> &out) {
    const long ori = r.l(), pad = r.l(), cur = r.l();
    const bool gridding = r.l() != 0;
    const int min_ires = (int)r.l();
    Projector P(ori, TRILINEAR, (float)pad, 10, 2);
    MultidimArray<RFLOAT> vol(ori, ori, ori), power;
    vol.setXmippOrigin();
    for (long n = 0; n < (long)MULTIDIM_SIZE(vol); ++n) vol.data[n] = r.d();
    P.computeFourierTransformMap(vol, power, cur, 1, gridding, true, min_ires);
    out.push_back(XSIZE(P.data));
    out.push_back(YSIZE(P.data));
    out.push_back(ZSIZE(P.data));
    out.push_back(STARTINGY(P.data));
    out.push_back(STARTINGZ(P.data));
    out.push_back(P.r_max);
    for (long n = 0; n < (long)MULTIDIM_SIZE(P.data); ++n) {
        out.push_back(P.data.data[n].real);
        out.push_back(P.data.data[n].imag);
    }
    for (long n = 0; n < (long)MULTIDIM_SIZE(power); ++n) out.push_back(power.data[n]);
}

}  // namespace

int main(int argc, char **argv) {
    if (argc != 4) {
        std::fprintf(stderr, "usage: ref_pin <mode> <request> <response>\n");
        return 2;
    }
    try {
        const std::vector<double> req = read_all(argv[2]);
        Reader r{req};
        std::vector<double> out;
        const std::string mode = argv[1];
        if (mode == "project") mode_project(r, out);
        else if (mode == "backproject") mode_backproject(r, out);
        else if (mode == "ctf") mode_ctf(r, out);
        else if (mode == "sampling") mode_sampling(r, out);
        else if (mode == "shift") mode_shift(r, out);
        else if (mode == "euler") mode_euler(r, out);
        else if (mode == "reconstruct") mode_reconstruct(r, out);
        else if (mode == "fouriermap") mode_fouriermap(r, out);
        else throw std::runtime_error("unknown mode " + mode);
        write_all(argv[3], out);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "ref_pin: %s\n", e.what());
        return 1;
    } catch (RelionError &e) {
        std::fprintf(stderr, "ref_pin: RelionError %s\n", e.msg.c_str());
        return 1;
    }
    return 0;
}
