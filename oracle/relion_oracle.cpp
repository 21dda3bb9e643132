/*
 * relion_oracle.cpp -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * A single-threaded, double-precision restatement of the CPU expectation
 * step of relion_refine (no --gpu, RFLOAT = double, exact Fourier shifts,
 * i.e. without --onthefly_shifts).  Each function cites the reference
 * file:line it follows.  The tests compare the CUDA path in
 * relion_gb300/csrc with it (test infrastructure); the product never links it.
 *
 * Scope (the configurations' case): one optics group whose pixel and box
 * size equal the model's, one image per particle, C1, NOPRIOR orientational
 * prior mode, no helical / multi-body / subtomogram / CC / gradient modes,
 * trilinear interpolation, no Ewald-sphere curvature, no anisotropic mag.
 *
 * Compile with -ffp-contract=off so that no multiply-add is fused: the
 * HEALPix and sampling arithmetic is compared bit-for-bit with the
 * reference's own code.
 */
#include "relion_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <omp.h>

namespace {

const double kPI = 3.14159265358979323846;          // src/macros.h:104
const double kHalfPi = 1.570796326794896619231321691639751442099;  // Healpix lsconstants.h:43
const double kEqualAccuracy = 1e-6;                  // src/macros.h:115 (double build)

// src/macros.h:197, :212, :226
inline int r_round(double x) { return (x > 0) ? (int)(x + 0.5) : (int)(x - 0.5); }
inline int r_ceil(double x) { return (x == (int)x) ? (int)x : ((x > 0) ? (int)(x + 1) : (int)x); }
inline int r_floor(double x) { return (x == (int)x) ? (int)x : ((x > 0) ? (int)x : (int)(x - 1)); }
inline double deg2rad(double d) { return d * kPI / 180; }   // src/macros.h:277
inline double rad2deg(double r) { return r * 180 / kPI; }   // src/macros.h:285

// ---------------------------------------------------------------------------
// HEALPix NEST scheme (Gorski et al. 2005), restated after the behaviour of
// src/Healpix_2.15a/healpix_base.cc:127-144 (nest2xyf/xyf2nest) and :494-527
// (pix2ang_z_phi, NEST branch).  Bit interleaving is done with plain loops.
// ---------------------------------------------------------------------------
struct Hpx {
    int order, nside, npface, npix;
    double fact1, fact2;
    explicit Hpx(int o) {
        order = o;
        nside = 1 << o;
        npface = nside << o;
        npix = 12 * npface;
        fact2 = 4. / npix;
        fact1 = (nside << 1) * fact2;
    }
};
const int kJrll[12] = {2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4};
const int kJpll[12] = {1, 3, 5, 7, 0, 2, 4, 6, 1, 3, 5, 7};

int deinterleave_even(int v) {  // bits 0,2,4,... -> 0,1,2,...
    int r = 0;
    for (int b = 0; b < 16; ++b) r |= ((v >> (2 * b)) & 1) << b;
    return r;
}
int interleave(int ix, int iy) {  // ix -> even bits, iy -> odd bits
    int r = 0;
    for (int b = 0; b < 16; ++b) r |= (((ix >> b) & 1) << (2 * b)) | (((iy >> b) & 1) << (2 * b + 1));
    return r;
}
void nest2xyf(const Hpx &h, int pix, int &ix, int &iy, int &face) {
    face = pix >> (2 * h.order);
    int p = pix & (h.npface - 1);
    ix = deinterleave_even(p);
    iy = deinterleave_even(p >> 1);
}
int xyf2nest(const Hpx &h, int ix, int iy, int face) {
    return (face << (2 * h.order)) + interleave(ix, iy);
}
void pix2ang_z_phi(const Hpx &h, int pix, double &z, double &phi) {
    int nl4 = h.nside * 4;
    int face, ix, iy;
    nest2xyf(h, pix, ix, iy, face);
    int jr = (kJrll[face] << h.order) - ix - iy - 1;
    int nr, kshift;
    if (jr < h.nside) {
        nr = jr;
        z = 1 - nr * nr * h.fact2;
        kshift = 0;
    } else if (jr > 3 * h.nside) {
        nr = nl4 - jr;
        z = nr * nr * h.fact2 - 1;
        kshift = 0;
    } else {
        nr = h.nside;
        z = (2 * h.nside - jr) * h.fact1;
        kshift = (jr - h.nside) & 1;
    }
    int jp = (kJpll[face] * nr + ix - iy + 1 + kshift) / 2;
    if (jp > nl4) jp -= nl4;
    if (jp < 1) jp += nl4;
    phi = (jp - (kshift + 1) * 0.5) * (kHalfPi / nr);
}

// src/healpix_sampling.cpp:1541-1564
void check_direction(double &rot, double &tilt) {
    if (tilt < 0.) {
        tilt = -tilt;
        rot += 180.;
    }
    for (;;) {
        if (rot > 180.) rot -= 360.;
        else if (rot < -180.) rot += 360.;
        else break;
    }
}
// src/healpix_sampling.cpp:1566-1577 (ACOSD as in src/macros.h:303)
void direction_from_pix(const Hpx &h, int ipix, double &rot, double &tilt) {
    double zz, phi;
    pix2ang_z_phi(h, ipix, zz, phi);
    rot = rad2deg(phi);
    tilt = acos(zz) * 180. / kPI;
    check_direction(rot, tilt);
}

// ---------------------------------------------------------------------------
// Sampling grid (HealpixSampling): C1 3D case, and the 2D (in-plane) case.
// ---------------------------------------------------------------------------
struct Sampling {
    bool is3d;
    int order;
    double psi_step;  // after rounding to 360/nr_psi (src/healpix_sampling.cpp:548-551)
    double offset_step, offset_range;  // Angstrom
    std::vector<double> rot, tilt;
    std::vector<int> ipix;
    std::vector<double> psi;
    std::vector<double> tx, ty;  // Angstrom
    Sampling(int order_, double psi_step_in, double range, double step, bool is3d_ = true) {
        is3d = is3d_;
        order = order_;
        // default psi step: src/healpix_sampling.cpp:71-76 (3D: HEALPix spacing; 2D: 10 degrees)
        double ps = psi_step_in;
        if (ps <= 0) ps = is3d ? 360. / (6 * r_round(std::pow(2., order))) : 10.;
        if (is3d) {
            Hpx h(order);
            // src/healpix_sampling.cpp:493-505 (C1: no symmetry-equivalent removal)
            for (int p = 0; p < h.npix; ++p) {
                double r, t;
                direction_from_pix(h, p, r, t);
                rot.push_back(r);
                tilt.push_back(t);
                ipix.push_back(p);
            }
        } else {
            // src/healpix_sampling.cpp:531-536: one direction, rot = tilt = 0
            rot.push_back(0.);
            tilt.push_back(0.);
            ipix.push_back(-1);
        }
        // src/healpix_sampling.cpp:544-555
        int nr_psi = r_ceil(360. / ps);
        psi_step = 360. / (double)nr_psi;
        for (int i = 0; i < nr_psi; ++i) psi.push_back(i * psi_step);
        // src/healpix_sampling.cpp:352-440 (2D translations, not helical)
        offset_range = range;
        offset_step = step;
        int maxp = r_ceil(offset_range / offset_step);
        for (long ix = -maxp; ix <= maxp; ++ix) {
            double xoff = ix * offset_step;
            for (long iy = -maxp; iy <= maxp; ++iy) {
                double yoff = iy * offset_step;
                double max2 = xoff * xoff + yoff * yoff;
                if (max2 < (offset_range * offset_range) + 0.001) {
                    tx.push_back(xoff);
                    ty.push_back(yoff);
                }
            }
        }
    }
    long ndir() const { return (long)rot.size(); }
    long npsi() const { return (long)psi.size(); }
    long ntrans() const { return (long)tx.size(); }
    // src/healpix_sampling.cpp:1644-1659
    int over_rot(int ov) const { return r_round(std::pow(2., ov * (is3d ? 3 : 1))); }
    static int over_trans(int ov) { return r_round(std::pow(2., ov * 2)); }

    // src/healpix_sampling.cpp:1832-1967 (no priors, no perturbation)
    void orientations(long idir, long ipsi, int ov, std::vector<double> &r, std::vector<double> &t,
                      std::vector<double> &p) const {
        r.clear(); t.clear(); p.clear();
        if (ov == 0) {
            r.push_back(rot[idir]);
            t.push_back(tilt[idir]);
            p.push_back(psi[ipsi]);
            return;
        }
        if (!is3d) {
            // src/healpix_sampling.cpp:1873-1877, 1951-1966: psi only, wrapped above 180
            int nr_ipsi_over = r_round(std::pow(2., ov));
            for (int k = 0; k < nr_ipsi_over; ++k) {
                double overpsi = psi[ipsi] - 0.5 * psi_step + (0.5 + k) * psi_step / nr_ipsi_over;
                if (overpsi > 180.) overpsi -= 360.;
                r.push_back(0.);
                t.push_back(0.);
                p.push_back(overpsi);
            }
            return;
        }
        Hpx base(order), over(order + ov);
        int fact = over.nside / base.nside;
        int x, y, face;
        nest2xyf(base, ipix[idir], x, y, face);
        int nr_ipsi_over = r_round(std::pow(2., ov));
        for (int j = fact * y; j < fact * (y + 1); ++j)
            for (int i = fact * x; i < fact * (x + 1); ++i) {
                int overpix = xyf2nest(over, i, j, face);
                double zz, phi;
                pix2ang_z_phi(over, overpix, zz, phi);
                double rr = rad2deg(phi);
                double tt = acos(zz) * 180. / kPI;
                check_direction(rr, tt);
                for (int k = 0; k < nr_ipsi_over; ++k) {
                    double overpsi = psi[ipsi] - 0.5 * psi_step + (0.5 + k) * psi_step / nr_ipsi_over;
                    r.push_back(rr);
                    t.push_back(tt);
                    p.push_back(overpsi);
                }
            }
    }
    // src/healpix_sampling.cpp:1724-1830 (2D, not helical, no perturbation)
    void translations_px(long itrans, int ov, double pix, std::vector<double> &x,
                         std::vector<double> &y) const {
        x.clear(); y.clear();
        if (ov == 0) {
            x.push_back(tx[itrans] / pix);
            y.push_back(ty[itrans] / pix);
            return;
        }
        int n = r_round(std::pow(2., ov));
        for (int ox = 0; ox < n; ++ox) {
            double ovx = tx[itrans] - 0.5 * offset_step + (0.5 + ox) * offset_step / n;
            for (int oy = 0; oy < n; ++oy) {
                double ovy = ty[itrans] - 0.5 * offset_step + (0.5 + oy) * offset_step / n;
                x.push_back(ovx / pix);
                y.push_back(ovy / pix);
            }
        }
    }
};

// src/euler.cpp:52-91
void euler_matrix(double alpha, double beta, double gamma, double A[9]) {
    alpha = deg2rad(alpha);
    beta = deg2rad(beta);
    gamma = deg2rad(gamma);
    double ca = cos(alpha), cb = cos(beta), cg = cos(gamma);
    double sa = sin(alpha), sb = sin(beta), sg = sin(gamma);
    double cc = cb * ca, cs = cb * sa, sc = sb * ca, ss = sb * sa;
    A[0] = cg * cc - sg * sa;
    A[1] = cg * cs + sg * ca;
    A[2] = -cg * sb;
    A[3] = -sg * cc - cg * sa;
    A[4] = -sg * cs + cg * ca;
    A[5] = sg * sb;
    A[6] = sc;
    A[7] = ss;
    A[8] = cb;
}

struct Cplx {
    double re, im;
};

// mymodel.prior_offset_class[iclass] (2D classification), zero when not given
double class_prior(const oracle_model &m, long iclass, int axis) {
    return m.prior_offset_class ? m.prior_offset_class[iclass * 2 + axis] : 0.;
}

// Fourier-slice projection: src/projector.cpp:630-733 (TRILINEAR branch).
// The inverse of the rotation is taken as its transpose (A.inv() in the
// reference; the two agree to rounding).  `out` is zero-filled first: points
// outside r_max stay zero, as in a freshly resized MultidimArray.
// Matrix2D<RFLOAT>::inv of a 3x3 matrix (src/matrix2d.h:1098-1125: the
// adjugate divided by the determinant, in the reference's order of
// operations), then *= padding factor (src/projector.cpp:638,
// src/backprojector.cpp:80-81).  The reference decides whether pixels exactly
// on the r_max circle are projected / inserted from this matrix in double
// precision, so the oracle uses the same matrix and the same tests.
void ref_inverse_pad(const double A[9], double pad, double Ai[9]) {
    const double a00 = A[0], a01 = A[1], a02 = A[2], a10 = A[3], a11 = A[4], a12 = A[5], a20 = A[6], a21 = A[7],
                 a22 = A[8];
    double r[9];
    r[0] = a22 * a11 - a21 * a12;
    r[1] = -(a22 * a01 - a21 * a02);
    r[2] = a12 * a01 - a11 * a02;
    r[3] = -(a22 * a10 - a20 * a12);
    r[4] = a22 * a00 - a20 * a02;
    r[5] = -(a12 * a00 - a10 * a02);
    r[6] = a21 * a10 - a20 * a11;
    r[7] = -(a21 * a00 - a20 * a01);
    r[8] = a11 * a00 - a10 * a01;
    const double tmp = a00 * r[0] + a10 * r[1] + a20 * r[2];
    for (int k = 0; k < 9; ++k) Ai[k] = (r[k] / tmp) * pad;
}

// The inverse-and-pad matrix of Projector::project (3D) / rotate2D (2D).
void projection_inverse(const oracle_model &m, const double A[9], double Ai[9]) {
    const double pad = (double)m.padding_factor;
    if (m.ref_dim == 2) {
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) Ai[r * 3 + c] = A[c * 3 + r] * pad;
    } else {
        ref_inverse_pad(A, pad, Ai);
    }
}

// One pixel (x, y) of Projector::project (3D, src/projector.cpp:664-733) or
// rotate2D (2D, :1048-1100) of class volume vol; false where the reference
// skips the pixel (radius test or outside the volume) and writes nothing.
bool project_pixel(const oracle_model &m, const Cplx *vol, const double Ai[9], int x, int y, Cplx &out) {
    const int r_max_ref = (int)(m.proj_r_max * m.padding_factor);
    const int r_max_ref_2 = r_max_ref * r_max_ref;
    const long xd = m.proj_xdim, yd = m.proj_ydim, zd = m.proj_zdim;
    double xp = Ai[0] * x + Ai[1] * y;
    double yp = Ai[3] * x + Ai[4] * y;
    double zp = Ai[6] * x + Ai[7] * y;
    if (m.ref_dim == 2) {
        // the radius test (:1055-1057) is made in integers as below
        if ((long)m.padding_factor * m.padding_factor * (x * x + y * y) > r_max_ref_2) return false;
        const bool neg2 = xp < 0;
        if (neg2) {
            xp = -xp;
            yp = -yp;
        }
        const int x0 = r_floor(xp);
        const double fx = xp - x0;
        int y0 = r_floor(yp);
        const double fy = yp - y0;
        y0 -= (int)m.proj_yinit;
        if (x0 < 0 || x0 + 1 >= xd || y0 < 0 || y0 + 1 >= yd) return false;
        auto at2 = [&](int yy, int xx) { return vol[(size_t)yy * xd + xx]; };
        auto lerp2 = [](double a, Cplx l, Cplx h) {  // LIN_INTERP, src/macros.h:373
            return Cplx{l.re + (h.re - l.re) * a, l.im + (h.im - l.im) * a};
        };
        Cplx dx0 = lerp2(fx, at2(y0, x0), at2(y0, x0 + 1));
        Cplx dx1 = lerp2(fx, at2(y0 + 1, x0), at2(y0 + 1, x0 + 1));
        Cplx v = lerp2(fy, dx0, dx1);
        if (neg2) v.im = -v.im;
        out = v;
        return true;
    }
    // r_ref_2 > r_max_ref_2 (:672), in double precision as the reference
    const double r_ref_2 = xp * xp + yp * yp + zp * zp;
    if (r_ref_2 > r_max_ref_2) return false;
    bool neg = (xp < 0);
    if (neg) {
        xp = -xp;
        yp = -yp;
        zp = -zp;
    }
    const int x0 = r_floor(xp);
    const double fx = xp - x0;
    const int x1 = x0 + 1;
    int y0 = r_floor(yp);
    const double fy = yp - y0;
    y0 -= (int)m.proj_yinit;
    const int y1 = y0 + 1;
    int z0 = r_floor(zp);
    const double fz = zp - z0;
    z0 -= (int)m.proj_zinit;
    const int z1 = z0 + 1;
    if (x0 < 0 || x0 + 1 >= xd || y0 < 0 || y0 + 1 >= yd || z0 < 0 || z0 + 1 >= zd) return false;
    auto at = [&](int zz, int yy, int xx) { return vol[((size_t)zz * yd + yy) * xd + xx]; };
    auto lerp = [](double a, Cplx l, Cplx h) {  // LIN_INTERP, src/macros.h:373
        return Cplx{l.re + (h.re - l.re) * a, l.im + (h.im - l.im) * a};
    };
    Cplx dx00 = lerp(fx, at(z0, y0, x0), at(z0, y0, x1));
    Cplx dx01 = lerp(fx, at(z1, y0, x0), at(z1, y0, x1));
    Cplx dx10 = lerp(fx, at(z0, y1, x0), at(z0, y1, x1));
    Cplx dx11 = lerp(fx, at(z1, y1, x0), at(z1, y1, x1));
    Cplx dxy0 = lerp(fy, dx00, dx10);
    Cplx dxy1 = lerp(fy, dx01, dx11);
    Cplx v = lerp(fz, dxy0, dxy1);
    if (neg) v.im = -v.im;
    out = v;
    return true;
}

const Cplx *class_volume(const oracle_model &m, long iclass) {
    return reinterpret_cast<const Cplx *>(m.ppref) + (size_t)iclass * m.proj_xdim * m.proj_ydim * m.proj_zdim;
}

// Projector::project / rotate2D of class iclass into out [size][size/2+1]:
// only the pixels inside the output image's circle (radius size / 2) that
// the reference does not skip are written; with clear, out is zeroed first
// (a fresh f2d), otherwise the other pixels keep their values, as the
// reference's projection buffer does between orientations.
void project(const oracle_model &m, long iclass, const double A[9], long size, Cplx *out, bool clear = true) {
    const long X = size / 2 + 1, Y = size;
    if (clear) std::memset(out, 0, sizeof(Cplx) * X * Y);
    double Ai[9];
    projection_inverse(m, A, Ai);
    const Cplx *vol = class_volume(m, iclass);
    const int r_max_out = (int)X - 1;
    const int r_max_out_2 = r_max_out * r_max_out;
    for (long i = 0; i < Y; ++i) {
        const int y = (i <= r_max_out) ? (int)i : (int)(i - Y);
        const int y2 = y * y;
        const int x_max = r_floor(std::sqrt((double)(r_max_out_2 - y2)));
        for (int x = 0; x <= x_max; ++x) {
            Cplx v;
            if (project_pixel(m, vol, Ai, x, y, v)) out[i * X + x] = v;
        }
    }
}

// The reference projects every orientation of one call of
// getAllSquaredDifferences or storeWeightedSums into one buffer (Fref,
// src/ml_optimiser.cpp:7269, 8431) that is never cleared between
// orientations: Projector::project does not zero its output
// (src/projector.cpp:632-634), so a pixel it skips for one orientation keeps
// the value of the last orientation that wrote it.  In 3D the only pixels
// skipped for some orientations and written for others are those exactly
// on the r_max circle, decided by the last bits of the rotated radius.
// StaleCircle records, along one call's sequence of projected orientations,
// the value each such pixel holds when an orientation skips it.
struct StaleCircle {
    std::vector<long> idx;  // flat index of each r_max-circle pixel in the image
    std::vector<int> xs, ys;
    std::vector<Cplx> last;
    std::vector<std::vector<std::pair<long, Cplx>>> patches;  // per sequence element

    StaleCircle(const oracle_model &m, long size) {
        if (m.ref_dim == 2) return;
        const long X = size / 2 + 1, Y = size;
        const int r_max_out = (int)X - 1, r2 = (int)(m.proj_r_max * m.proj_r_max);
        for (long i = 0; i < Y; ++i) {
            const int y = (i <= r_max_out) ? (int)i : (int)(i - Y);
            const int x_max = r_floor(std::sqrt((double)(r_max_out * r_max_out - y * y)));
            for (int x = 0; x <= x_max; ++x)
                if (x * x + y * y == r2) {
                    idx.push_back(i * X + x);
                    xs.push_back(x);
                    ys.push_back(y);
                }
        }
        last.assign(idx.size(), Cplx{0, 0});
    }
    // the next orientation of the sequence: returns its element index
    long add(const oracle_model &m, long iclass, const double A[9]) {
        patches.emplace_back();
        if (idx.empty()) return (long)patches.size() - 1;
        double Ai[9];
        projection_inverse(m, A, Ai);
        const Cplx *vol = class_volume(m, iclass);
        for (size_t c = 0; c < idx.size(); ++c) {
            Cplx v;
            if (project_pixel(m, vol, Ai, xs[c], ys[c], v))
                last[c] = v;
            else
                patches.back().push_back({idx[c], last[c]});
        }
        return (long)patches.size() - 1;
    }
    void apply(long e, Cplx *out) const {
        for (const auto &pv : patches[(size_t)e]) out[pv.first] = pv.second;
    }
};

// Trilinear insertion: src/backprojector.cpp:55-296 (no Ewald sphere,
// identity magnification).  Data/weight accumulate in double.
void backproject(const oracle_model &m, long iclass, const double A[9], long size, const Cplx *f2d,
                 const double *Mw, double *bp_data, double *bp_weight) {
    const double pad = (double)m.padding_factor;
    double Ai[9];
    if (m.ref_dim == 2) {
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) Ai[r * 3 + c] = A[c * 3 + r] * pad;
    } else {
        ref_inverse_pad(A, pad, Ai);
    }
    const int max_r2 = r_round(m.bp_r_max * pad) * r_round(m.bp_r_max * pad);
    // the ellipse |Ainv (x, y)|^2 <= max_r2 bounding x per row (:84-92, :150-160)
    const double AtA_xx = Ai[0] * Ai[0] + Ai[3] * Ai[3] + Ai[6] * Ai[6];
    const double AtA_xy = Ai[0] * Ai[1] + Ai[3] * Ai[4] + Ai[6] * Ai[7];
    const double AtA_yy = Ai[1] * Ai[1] + Ai[4] * Ai[4] + Ai[7] * Ai[7];
    const double AtA_xy2 = AtA_xy * AtA_xy;
    const long s = size, sh = size / 2 + 1;
    const long xd = m.bp_xdim, yd = m.bp_ydim, zd = m.bp_zdim;
    const size_t vox = (size_t)xd * yd * zd;
    Cplx *data = reinterpret_cast<Cplx *>(bp_data) + (size_t)iclass * vox;
    double *weight = bp_weight + (size_t)iclass * vox;
    for (long i = 0; i < s; ++i) {
        int y, first_allowed_x;
        if (i < sh) {
            y = (int)i;
            first_allowed_x = 0;
        } else {
            y = (int)(i - s);
            first_allowed_x = 1;
        }
        // x bounded by the ellipse of this row (:150-160) and r2_3D > max_r2
        // re-checked per pixel (:188), in double precision as the reference;
        // 2D: the integer circle test of backrotate2D
        int first_x = first_allowed_x, last_x = (int)(sh - 1);
        if (m.ref_dim != 2) {
            const double discr = AtA_xy2 * y * y - AtA_xx * (AtA_yy * y * y - max_r2);
            if (discr < 0.) continue;
            const double d = std::sqrt(discr) / AtA_xx;
            const double q = -AtA_xy * y / AtA_xx;
            first_x = std::max(first_x, r_ceil(q - d));
            last_x = std::min(last_x, r_floor(q + d));
        }
        for (int x = first_x; x <= last_x; ++x) {
            if (m.ref_dim == 2 &&
                (long)m.padding_factor * m.padding_factor * ((long)x * x + (long)y * y) > max_r2)
                continue;
            Cplx val = f2d[i * sh + x];
            double w = Mw[i * sh + x];
            if (w <= 0.) continue;
            double xp = Ai[0] * x + Ai[1] * y;
            double yp = Ai[3] * x + Ai[4] * y;
            double zp = Ai[6] * x + Ai[7] * y;
            if (m.ref_dim != 2 && xp * xp + yp * yp + zp * zp > max_r2) continue;
            bool neg = xp < 0;
            if (neg) {
                xp = -xp;
                yp = -yp;
                zp = -zp;
            }
            int x0 = r_floor(xp);
            double fx = xp - x0;
            int x1 = x0 + 1;
            int y0 = r_floor(yp);
            double fy = yp - y0;
            y0 -= (int)m.bp_yinit;
            int y1 = y0 + 1;
            if (m.ref_dim == 2) {
                // BackProjector::backrotate2D (src/backprojector.cpp:471-660):
                // bilinear insertion into the 2D data / weight planes
                if (x0 < 0 || x0 + 1 >= xd || y0 < 0 || y0 + 1 >= yd) continue;
                const double mx = 1. - fx, my = 1. - fy;
                const double d4[4] = {my * mx, my * fx, fy * mx, fy * fx};
                if (neg) val.im = -val.im;
                const int ys4[4] = {y0, y0, y1, y1}, xs4[4] = {x0, x1, x0, x1};
                for (int c = 0; c < 4; ++c) {
                    size_t idx = (size_t)ys4[c] * xd + xs4[c];
                    data[idx].re += d4[c] * val.re;
                    data[idx].im += d4[c] * val.im;
                    weight[idx] += d4[c] * w;
                }
                continue;
            }
            int z0 = r_floor(zp);
            double fz = zp - z0;
            z0 -= (int)m.bp_zinit;
            int z1 = z0 + 1;
            if (x0 < 0 || x0 + 1 >= xd || y0 < 0 || y0 + 1 >= yd || z0 < 0 || z0 + 1 >= zd) continue;
            double mfx = 1. - fx, mfy = 1. - fy, mfz = 1. - fz;
            double dd[8] = {mfz * mfy * mfx, mfz * mfy * fx, mfz * fy * mfx, mfz * fy * fx,
                            fz * mfy * mfx,  fz * mfy * fx,  fz * fy * mfx,  fz * fy * fx};
            if (neg) val.im = -val.im;
            int zs[8] = {z0, z0, z0, z0, z1, z1, z1, z1};
            int ys[8] = {y0, y0, y1, y1, y0, y0, y1, y1};
            int xs[8] = {x0, x1, x0, x1, x0, x1, x0, x1};
            for (int c = 0; c < 8; ++c) {
                size_t idx = ((size_t)zs[c] * yd + ys[c]) * xd + xs[c];
                data[idx].re += dd[c] * val.re;
                data[idx].im += dd[c] * val.im;
                weight[idx] += dd[c] * w;
            }
        }
    }
}

// Crop (window) an FFTW half-transform to a smaller size:
// src/fftw.h:809-857 (newhdim <= XSIZE(in) branch).
std::vector<Cplx> window_ft(const Cplx *in, long in_size, long out_size) {
    long Xi = in_size / 2 + 1, Xo = out_size / 2 + 1;
    std::vector<Cplx> out((size_t)out_size * Xo, Cplx{0, 0});
    for (long i = 0; i < out_size; ++i) {
        long ip = (i < Xo) ? i : i - out_size;
        long ii = (ip < 0) ? ip + in_size : ip;
        for (long j = 0; j < Xo; ++j) out[i * Xo + j] = in[ii * Xi + j];
    }
    return out;
}
std::vector<double> window_real(const double *in, long in_size, long out_size) {
    long Xi = in_size / 2 + 1, Xo = out_size / 2 + 1;
    std::vector<double> out((size_t)out_size * Xo, 0.);
    for (long i = 0; i < out_size; ++i) {
        long ip = (i < Xo) ? i : i - out_size;
        long ii = (ip < 0) ? ip + in_size : ip;
        for (long j = 0; j < Xo; ++j) out[i * Xo + j] = in[ii * Xi + j];
    }
    return out;
}

// Exact phase shift: src/fftw.cpp:842-920 (2D branch).
void shift_ft(const Cplx *in, long size, double oridim, double xshift, double yshift, Cplx *out) {
    long X = size / 2 + 1, Y = size;
    xshift /= -oridim;
    yshift /= -oridim;
    if (std::fabs(xshift) < kEqualAccuracy && std::fabs(yshift) < kEqualAccuracy) {
        std::memcpy(out, in, sizeof(Cplx) * X * Y);
        return;
    }
    for (long i = 0; i < Y; ++i) {
        double y = (i < X) ? (double)i : (double)(i - Y);
        for (long j = 0; j < X; ++j) {
            double x = (double)j;
            double dotp = 2 * kPI * (x * xshift + y * yshift);
            double b = sin(dotp), a = cos(dotp);
            double c = in[i * X + j].re, d = in[i * X + j].im;
            double ac = a * c, bd = b * d, ab_cd = (a + b) * (c + d);
            out[i * X + j] = Cplx{ac - bd, ab_cd - ac - bd};
        }
    }
}

// Resolution-shell index per Fourier pixel: src/ml_optimiser.cpp:5784-5795
std::vector<int> mresol(long size) {
    long X = size / 2 + 1;
    std::vector<int> r((size_t)size * X, -1);
    for (long i = 0; i < size; ++i) {
        long ip = (i < X) ? i : i - size;
        for (long j = 0; j < X; ++j) {
            int ires = r_round(std::sqrt((double)(ip * ip + j * j)));
            if (ires < size / 2 + 1 && !(j == 0 && ip < 0)) r[i * X + j] = ires;
        }
    }
    return r;
}

// Minvsigma2: src/ml_optimiser.cpp:6880-6892 (remap factor 1).
std::vector<double> minvsigma2(const oracle_model &m, const std::vector<int> &res) {
    std::vector<double> v(res.size(), 0.);
    for (size_t n = 0; n < res.size(); ++n) {
        int ires = res[n];
        int ires_remapped = r_round(1.0 * ires);
        if (ires > 0 && ires_remapped < m.sigma2_len)
            v[n] = 1. / (m.sigma2_fudge * m.sigma2_noise[ires_remapped]);
    }
    return v;
}

struct PassOut {
    std::vector<double> Mweight;  // diff2, then weights
    double min_diff2;
};

}  // namespace

extern "C" {

/* Host threads of the oracle's parallel loops (omp_set_num_threads on the
 * calling thread, which is what counts even when the OpenMP runtime was
 * started earlier by another library); returns the number now in effect. */
int oracle_set_threads(int n) {
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
}

double oracle_ctf(double defU, double defV, double defAng, double kV, double Cs, double Q0,
                  double Bfac, double scale, double phase_shift, double X, double Y) {
    // src/ctf.cpp:211-261 (initialise) and src/ctf.h:184-256 (getCTF, damping on)
    double local_Cs = Cs * 1e7, local_kV = kV * 1e3;
    double rad_az = deg2rad(defAng);
    double lambda = 12.2643247 / std::sqrt(local_kV * (1. + local_kV * 0.978466e-6));
    double K1 = kPI / 2 * 2 * lambda;
    double K2 = kPI / 2 * local_Cs * lambda * lambda * lambda;
    double K3 = std::atan(Q0 / std::sqrt(1 - Q0 * Q0));
    double K4 = -Bfac / 4.;
    double K5 = deg2rad(phase_shift);
    double s = std::sin(rad_az), c = std::cos(rad_az);
    // A = (Q^T D) Q with Q = [[c, s], [-s, c]], D = diag(-defU, -defV),
    // multiplied in that order as the reference's 2x2 products do
    // (src/ctf.cpp:251-257; src/jaz/gravis/t2Matrix.h operator*)
    const double M00 = c * (-defU), M01 = (-s) * (-defV), M10 = s * (-defU), M11 = c * (-defV);
    double Axx = M00 * c + M01 * (-s);
    double Axy = M00 * s + M01 * c;
    double Ayy = M10 * s + M11 * c;
    double u2 = X * X + Y * Y, u4 = u2 * u2;
    double gamma = K1 * (Axx * X * X + 2.0 * Axy * X * Y + Ayy * Y * Y) + K2 * u4 - K5 - K3;
    double ret = -std::sin(gamma);
    ret *= std::exp(K4 * u2);
    ret *= scale;
    if (std::fabs(ret) < 1e-8) ret = (ret < 0 ? -1. : 1.) * 1e-8;
    return ret;
}

int oracle_sampling_sizes(int64_t order, double psi_step, double offset_range, double offset_step,
                          int64_t *ndir, int64_t *npsi, int64_t *ntrans) {
    Sampling s((int)order, psi_step, offset_range, offset_step);
    *ndir = s.ndir();
    *npsi = s.npsi();
    *ntrans = s.ntrans();
    return 0;
}

int oracle_directions(int64_t order, double *rot, double *tilt, int64_t *ipix) {
    Sampling s((int)order, 10., 1., 1.);
    for (long i = 0; i < s.ndir(); ++i) {
        rot[i] = s.rot[i];
        tilt[i] = s.tilt[i];
        ipix[i] = s.ipix[i];
    }
    return 0;
}

int oracle_oversampled_orientations(int64_t order, double psi_step, int64_t idir, int64_t ipsi,
                                    int64_t ov, double *rot, double *tilt, double *psi) {
    Sampling s((int)order, psi_step, 1., 1.);
    std::vector<double> r, t, p;
    s.orientations(idir, ipsi, (int)ov, r, t, p);
    for (size_t i = 0; i < r.size(); ++i) {
        rot[i] = r[i];
        tilt[i] = t[i];
        psi[i] = p[i];
    }
    return (int)r.size();
}

int oracle_translations(double offset_range, double offset_step, double *tx, double *ty) {
    Sampling s(0, 10., offset_range, offset_step);
    for (long i = 0; i < s.ntrans(); ++i) {
        tx[i] = s.tx[i];
        ty[i] = s.ty[i];
    }
    return (int)s.ntrans();
}

int oracle_oversampled_translations(double offset_range, double offset_step, int64_t itrans,
                                    int64_t ov, double pixel_size, double *tx, double *ty) {
    Sampling s(0, 10., offset_range, offset_step);
    std::vector<double> x, y;
    s.translations_px(itrans, (int)ov, pixel_size, x, y);
    for (size_t i = 0; i < x.size(); ++i) {
        tx[i] = x[i];
        ty[i] = y[i];
    }
    return (int)x.size();
}

void oracle_hpx_pix2ang_z_phi(int64_t order, int64_t pix, double *z, double *phi) {
    Hpx h((int)order);
    pix2ang_z_phi(h, (int)pix, *z, *phi);
}
void oracle_hpx_nest2xyf(int64_t order, int64_t pix, int64_t *ix, int64_t *iy, int64_t *face) {
    Hpx h((int)order);
    int a, b, f;
    nest2xyf(h, (int)pix, a, b, f);
    *ix = a;
    *iy = b;
    *face = f;
}
int64_t oracle_hpx_xyf2nest(int64_t order, int64_t ix, int64_t iy, int64_t face) {
    Hpx h((int)order);
    return xyf2nest(h, (int)ix, (int)iy, (int)face);
}
void oracle_euler(double rot, double tilt, double psi, double *A) { euler_matrix(rot, tilt, psi, A); }

void oracle_project(const oracle_model *m, int64_t iclass, const double *A, int64_t size, double *out) {
    project(*m, iclass, A, size, reinterpret_cast<Cplx *>(out));
}

void oracle_backproject(const oracle_model *m, int64_t iclass, const double *A, int64_t size, const double *f2d,
                        const double *Mw, double *bp_data, double *bp_weight) {
    backproject(*m, iclass, A, size, reinterpret_cast<const Cplx *>(f2d), Mw, bp_data, bp_weight);
}

void oracle_shift_ft(const double *in, int64_t size, double oridim, double xshift, double yshift, double *out) {
    shift_ft(reinterpret_cast<const Cplx *>(in), size, oridim, xshift, yshift, reinterpret_cast<Cplx *>(out));
}

/*
 * The expectation step for n particles: src/ml_optimiser.cpp:4376-4700
 * (expectationOneParticle), calling getAllSquaredDifferences (:7098),
 * convertAllSquaredDifferencesToWeights (:7704) and storeWeightedSums (:8241).
 */
int oracle_expectation(const oracle_model *mp, int64_t n, const oracle_particle *parts,
                       oracle_result *res, oracle_debug *dbg, oracle_wsum *wsum) {
    const oracle_model &m = *mp;
    const bool is2d = m.ref_dim == 2;
    Sampling S((int)m.healpix_order, m.psi_step, m.offset_range, m.offset_step, !is2d);
    const long K = m.nr_classes, ND = S.ndir(), NP = S.npsi(), NT = S.ntrans();
    const int ov = (int)m.adaptive_oversampling;
    const long nOR = S.over_rot(ov), nOT = Sampling::over_trans(ov);
    const long R = K * ND * NP;
    const long cur = m.current_size, crs = m.coarse_size;
    const long Xf = cur / 2 + 1;
    const long npix_f = cur * Xf;
    const double pix = m.pixel_size;
    const std::vector<int> Mres_c = mresol(crs), Mres_f = mresol(cur);
    const std::vector<double> inv_c = minvsigma2(m, Mres_c), inv_f = minvsigma2(m, Mres_f);
    const long nhalf = m.ori_size / 2 + 1;

    for (long ip = 0; ip < n; ++ip) {
        const oracle_particle &P = parts[ip];
        const Cplx *Fimg_f = reinterpret_cast<const Cplx *>(P.fimg);
        const Cplx *Fnm_f = reinterpret_cast<const Cplx *>(P.fimg_nomask);
        std::vector<Cplx> Fimg_c = window_ft(Fimg_f, cur, crs);
        std::vector<double> Fctf_c = window_real(P.fctf, cur, crs);
        const double myscale_d2 = m.do_scale_correction ? P.scale : 1.0;

        double sig_weight = -1.;
        std::vector<uint8_t> coarse_sig;
        std::vector<double> Mw;       // exp_Mweight of the current pass
        double min_diff2 = 0, sum_weight = 0;
        long nr_sign = 0;

        for (int ipass = 0; ipass < 2; ++ipass) {
            const int cov = ipass == 0 ? 0 : ov;
            const long size = ipass == 0 ? crs : cur;
            const long X = size / 2 + 1, npix = size * X;
            const Cplx *Fimg = ipass == 0 ? Fimg_c.data() : Fimg_f;
            const double *Fctf = ipass == 0 ? Fctf_c.data() : P.fctf;
            const std::vector<double> &inv = ipass == 0 ? inv_c : inv_f;
            const long nor = ipass == 0 ? 1 : nOR, not_ = ipass == 0 ? 1 : nOT;

            // shifted images: precalculateShiftedImagesCtfsAndInvSigma2s (:6755)
            std::vector<std::vector<Cplx>> shifted((size_t)NT * not_, std::vector<Cplx>(npix));
            std::vector<double> sx, sy;
            for (long it = 0; it < NT; ++it) {
                S.translations_px(it, cov, pix, sx, sy);
                for (long io = 0; io < not_; ++io)
                    shift_ft(Fimg, size, (double)m.ori_size, sx[io], sy[io], shifted[it * not_ + io].data());
            }

            // getAllSquaredDifferences (:7098-7700)
            const long nW = R * NT * nor * not_;
            Mw.assign(nW, -999.);
            min_diff2 = 99e99;  // LARGE_NUMBER, src/macros.h:78
            // orientations are independent: threads split (class, direction,
            // psi); each writes its own hidden indices and a private minimum.
            // The reference projects them in this order into one buffer; the
            // values it leaves at skipped r_max-circle pixels are found first
            // along that order (StaleCircle).
            const long n_orient = K * ND * NP;
            StaleCircle stale(m, size);
            std::vector<long> elem_of(n_orient, -1);
            {
                std::vector<double> ro, ti, ps;
                double A[9];
                for (long ioc = 0; ioc < n_orient; ++ioc) {
                    const long ic = ioc / (ND * NP), id = (ioc / NP) % ND, is = ioc % NP;
                    if (!(m.pdf_class[ic] > 0.)) continue;
                    bool proceed = true;
                    if (ipass > 0) {
                        proceed = false;
                        for (long it = 0; it < NT; ++it)
                            if (coarse_sig[ioc * NT + it]) { proceed = true; break; }
                    }
                    if (!(proceed && m.pdf_direction[ic * ND + id] > 0.)) continue;
                    S.orientations(id, is, cov, ro, ti, ps);
                    for (long ior = 0; ior < nor; ++ior) {
                        euler_matrix(ro[ior], ti[ior], ps[ior], A);
                        const long e = stale.add(m, ic, A);
                        if (ior == 0) elem_of[ioc] = e;
                    }
                }
            }
#pragma omp parallel
            {
                std::vector<Cplx> Fref(npix), Frefctf(npix);
                std::vector<double> ro, ti, ps;
                double A[9];
                double my_min = 99e99;
#pragma omp for schedule(dynamic, 4)
                for (long ioc = 0; ioc < n_orient; ++ioc) {
                    const long ic = ioc / (ND * NP), id = (ioc / NP) % ND, is = ioc % NP;
                    if (!(m.pdf_class[ic] > 0.)) continue;
                    double pdf_orient = m.pdf_direction[ic * ND + id];
                    bool proceed = true;
                    if (ipass > 0) {
                        proceed = false;
                        for (long it = 0; it < NT; ++it)
                            if (coarse_sig[ioc * NT + it]) { proceed = true; break; }
                    }
                    if (!(proceed && pdf_orient > 0.)) continue;
                    S.orientations(id, is, cov, ro, ti, ps);
                    for (long ior = 0; ior < nor; ++ior) {
                        euler_matrix(ro[ior], ti[ior], ps[ior], A);
                        project(m, ic, A, size, reinterpret_cast<Cplx *>(Fref.data()));
                        stale.apply(elem_of[ioc] + ior, Fref.data());
                        for (long k = 0; k < npix; ++k) {
                            Frefctf[k].re = Fref[k].re * Fctf[k] * myscale_d2;
                            Frefctf[k].im = Fref[k].im * Fctf[k] * myscale_d2;
                        }
                        for (long it = 0; it < NT; ++it) {
                            long ihidden = ioc * NT + it;
                            if (ipass > 0 && !coarse_sig[ihidden]) continue;
                            for (long io = 0; io < not_; ++io) {
                                long iho = ipass == 0 ? ihidden : ihidden * nor * not_ + ior * not_ + io;
                                const Cplx *Fs = shifted[it * not_ + io].data();
                                double diff2 = P.highres_Xi2 / 2.;
                                for (long k = 0; k < npix; ++k) {
                                    double dr = Frefctf[k].re - Fs[k].re;
                                    double di = Frefctf[k].im - Fs[k].im;
                                    diff2 += (dr * dr + di * di) * 0.5 * inv[k];
                                }
                                Mw[iho] = diff2;  // single image: first write
                                if (diff2 < my_min) my_min = diff2;
                            }
                        }
                    }
                }
#pragma omp critical
                if (my_min < min_diff2) min_diff2 = my_min;
            }
            if (dbg) {
                double *dst = ipass == 0 ? dbg[ip].coarse_diff2 : dbg[ip].fine_diff2;
                if (dst) std::memcpy(dst, Mw.data(), sizeof(double) * nW);
            }

            // convertAllSquaredDifferencesToWeights (:7704-8239), NOPRIOR
            double s2x = m.sigma2_offset, s2y = m.sigma2_offset;
            double offset_norm = 2. * kPI * std::sqrt(s2x) * std::sqrt(s2y);
            double pdf_orient_mean = 0, pdf_offset_mean = 0;
            unsigned long orient_count = 0, offset_count = 0;
            // 2D: the offset prior is the class's (mymodel.prior_offset_class, :7829-7833)
            std::vector<double> tdiff2s((size_t)K * NT);
            for (long ic = 0; ic < K; ++ic) {
                const double prx = is2d ? class_prior(m, ic, 0) : P.prior[0];
                const double pry = is2d ? class_prior(m, ic, 1) : P.prior[1];
                for (long id = 0; id < ND; ++id)
                    for (long is = 0; is < NP; ++is) {
                        pdf_orient_mean += m.pdf_direction[ic * ND + id];
                        orient_count++;
                    }
                for (long it = 0; it < NT; ++it) {
                    double ox = P.old_offset[0] + S.tx[it];
                    double oy = P.old_offset[1] + S.ty[it];
                    double td = 0.;
                    td += (ox - prx) * (ox - prx) / (-2. * s2x);
                    td += (oy - pry) * (oy - pry) / (-2. * s2y);
                    td *= pix * pix;
                    tdiff2s[ic * NT + it] = td;
                    if (s2x < 0.0001) pdf_offset_mean += (td > 0.) ? 0. : 1.;
                    else pdf_offset_mean += std::exp(td) / offset_norm;
                    offset_count++;
                }
            }
            pdf_orient_mean /= (double)orient_count;
            pdf_offset_mean /= (double)offset_count;
            sum_weight = 0.;
            for (long ic = 0; ic < K; ++ic)
                for (long id = 0; id < ND; ++id)
                    for (long is = 0; is < NP; ++is) {
                        long ioc = ic * ND * NP + id * NP + is;
                        double pdf_orient = m.pdf_direction[ic * ND + id];
                        if (pdf_orient_mean != 0.) pdf_orient /= pdf_orient_mean;
                        for (long it = 0; it < NT; ++it) {
                            double td = tdiff2s[ic * NT + it];
                            double pdf_offset;
                            if (s2x < 0.0001) pdf_offset = (td > 0.) ? 0. : 1.;
                            else pdf_offset = std::exp(td) / offset_norm;
                            if (pdf_offset_mean > 0.) pdf_offset /= pdf_offset_mean;
                            long iho = (ioc * NT + it) * nor * not_;
                            for (long k = 0; k < nor * not_; ++k, ++iho) {
                                if (Mw[iho] < 0.) {
                                    Mw[iho] = 0.;
                                } else {
                                    double w = pdf_orient * pdf_offset;
                                    double d = Mw[iho] - min_diff2;
                                    if (d > 700.) w = 0.;
                                    else w *= std::exp(-d);
                                    Mw[iho] = w;
                                    sum_weight += w;
                                }
                            }
                        }
                    }
            if (sum_weight == 0. || std::isnan(sum_weight)) return -1;  // "zero sum of weights"
            // significance (:8120-8200)
            std::vector<double> sorted;
            sorted.reserve(nW);
            for (long i = 0; i < nW; ++i)
                if (Mw[i] > 0.) sorted.push_back(Mw[i]);
            if (sorted.empty()) return -2;
            std::sort(sorted.begin(), sorted.end());
            double frac = 0., my_sig = 0.;
            long my_nr = 0;
            for (long i = (long)sorted.size() - 1; i >= 0; --i) {
                if (m.maximum_significants > 0) {
                    if (my_nr < m.maximum_significants) {
                        if (ipass == 0) my_nr++;
                        my_sig = sorted[i];
                    }
                } else {
                    if (ipass == 0) my_nr++;
                    my_sig = sorted[i];
                }
                frac += sorted[i];
                if (frac > m.adaptive_fraction * sum_weight) break;
            }
            if (ipass == 0 && my_nr == 0) return -3;
            if (ipass == 0) {
                nr_sign = my_nr;
                coarse_sig.assign(nW, 0);
                for (long i = 0; i < nW; ++i) coarse_sig[i] = (Mw[i] >= my_sig) ? 1 : 0;
                res[ip].coarse_min_diff2 = min_diff2;
                res[ip].coarse_sum_weight = sum_weight;
                res[ip].coarse_significant_weight = my_sig;
                if (dbg) {
                    if (dbg[ip].coarse_weight) std::memcpy(dbg[ip].coarse_weight, Mw.data(), sizeof(double) * nW);
                    if (dbg[ip].coarse_significant) std::memcpy(dbg[ip].coarse_significant, coarse_sig.data(), nW);
                }
            } else {
                res[ip].fine_min_diff2 = min_diff2;
                res[ip].fine_sum_weight = sum_weight;
                res[ip].fine_significant_weight = my_sig;
                if (dbg && dbg[ip].fine_weight) std::memcpy(dbg[ip].fine_weight, Mw.data(), sizeof(double) * nW);
            }
            sig_weight = my_sig;
        }

        // ---- storeWeightedSums (:8241-9157) -------------------------------
        const long X = Xf, npix = npix_f;
        std::vector<double> Minv(npix, 1.);
        std::vector<double> inv_store = inv_f;
        inv_store[0] = 1. / (m.sigma2_fudge * m.sigma2_noise[0]);  // :8301
        if (m.do_map) Minv = inv_store;
        std::vector<std::vector<Cplx>> sh_m((size_t)NT * nOT, std::vector<Cplx>(npix));
        std::vector<std::vector<Cplx>> sh_n((size_t)NT * nOT, std::vector<Cplx>(npix));
        std::vector<double> sx, sy;
        std::vector<std::vector<double>> otx(NT), oty(NT);
        for (long it = 0; it < NT; ++it) {
            S.translations_px(it, ov, pix, sx, sy);
            otx[it] = sx;
            oty[it] = sy;
            for (long io = 0; io < nOT; ++io) {
                shift_ft(Fimg_f, cur, (double)m.ori_size, sx[io], sy[io], sh_m[it * nOT + io].data());
                shift_ft(Fnm_f, cur, (double)m.ori_size, sx[io], sy[io], sh_n[it * nOT + io].data());
            }
        }
        std::vector<double> thr_sigma2(nhalf, 0.);
        double norm_corr = 0., XA = 0., AA = 0., sumw_group = 0., sigma2_off = 0.;
        std::vector<double> thr_pdf_class(K, 0.), thr_pdf_dir(K * ND, 0.), thr_prior_off(2 * K, 0.);
        double max_weight = -1.;
        std::vector<Cplx> Fref(npix), Frefctf(npix), Fimg(npix);
        std::vector<double> Mctf(npix), Fweight(npix);
        std::vector<double> ro, ti, ps;
        double A[9];
        const double *dvp = m.data_vs_prior;
        for (long ic = 0; ic < K; ++ic)
            for (long id = 0; id < ND; ++id)
                for (long is = 0; is < NP; ++is) {
                    long ioc = ic * ND * NP + id * NP + is;
                    bool any = false;
                    for (long it = 0; it < NT; ++it)
                        if (coarse_sig[ioc * NT + it]) { any = true; break; }
                    if (!any) continue;
                    S.orientations(id, is, ov, ro, ti, ps);
                    for (long ior = 0; ior < nOR; ++ior) {
                        euler_matrix(ro[ior], ti[ior], ps[ior], A);
                        // one buffer along the loop, as the reference's Fref
                        project(m, ic, A, cur, Fref.data(), false);
                        std::fill(Fimg.begin(), Fimg.end(), Cplx{0, 0});
                        std::fill(Fweight.begin(), Fweight.end(), 0.);
                        double myscale = 1.;
                        if (m.do_scale_correction) {
                            myscale = P.scale;
                            if (myscale < 0.001) myscale = 0.001;
                        }
                        for (long k = 0; k < npix; ++k) {
                            Mctf[k] = P.fctf[k] * myscale;
                            Frefctf[k].re = Fref[k].re * P.fctf[k] * myscale;
                            Frefctf[k].im = Fref[k].im * P.fctf[k] * myscale;
                        }
                        for (long it = 0, iit = 0; it < NT; ++it) {
                            long ihidden = ioc * NT + it;
                            for (long io = 0; io < nOT; ++io, ++iit) {
                                long iho = ihidden * nOT * nOR + ior * nOT + io;
                                double w = Mw[iho];
                                if (!(w >= sig_weight)) continue;
                                w /= sum_weight;
                                const Cplx *Fs = sh_m[iit].data();
                                const Cplx *Fn = sh_n[iit].data();
                                for (long k = 0; k < npix; ++k) {
                                    int ires = Mres_f[k];
                                    if (ires > -1) {
                                        double dr = Frefctf[k].re - Fs[k].re;
                                        double di = Frefctf[k].im - Fs[k].im;
                                        double wd = w * (dr * dr + di * di);
                                        thr_sigma2[ires] += wd;
                                        norm_corr += wd;
                                        if (m.do_scale_correction && dvp[ic * nhalf + ires] > 3.) {
                                            XA += w * (Frefctf[k].re * Fs[k].re + Frefctf[k].im * Fs[k].im);
                                            AA += w * (Frefctf[k].re * Frefctf[k].re + Frefctf[k].im * Frefctf[k].im);
                                        }
                                    }
                                }
                                sumw_group += w;
                                thr_pdf_class[ic] += w;
                                // 2D: class offset prior and its weighted sum (:8449-8456, :8668-8672)
                                const double prx = is2d ? class_prior(m, ic, 0) : P.prior[0];
                                const double pry = is2d ? class_prior(m, ic, 1) : P.prior[1];
                                double dx = prx - P.old_offset[0] - otx[it][io];
                                double dy = pry - P.old_offset[1] - oty[it][io];
                                sigma2_off += w * pix * pix * dx * dx;
                                sigma2_off += w * pix * pix * dy * dy;
                                if (is2d) {
                                    thr_prior_off[ic * 2 + 0] += w * pix * (P.old_offset[0] + otx[it][io]);
                                    thr_prior_off[ic * 2 + 1] += w * pix * (P.old_offset[1] + oty[it][io]);
                                }
                                thr_pdf_dir[ic * ND + id] += w;
                                for (long k = 0; k < npix; ++k) {
                                    double wis = w * Mctf[k] * Minv[k];
                                    Fimg[k].re += Fn[k].re * wis;
                                    Fimg[k].im += Fn[k].im * wis;
                                    Fweight[k] += wis * Mctf[k];
                                }
                                if (w > max_weight) {
                                    max_weight = w;
                                    res[ip].rot = ro[ior];
                                    res[ip].tilt = ti[ior];
                                    res[ip].psi = ps[ior];
                                    res[ip].xoff = P.old_offset[0] + otx[it][io];
                                    res[ip].yoff = P.old_offset[1] + oty[it][io];
                                    res[ip].cls = (double)ic + 1;
                                    res[ip].pmax = max_weight;
                                    res[ip].best_ihidden_over = iho;
                                }
                            }
                        }
                        if (wsum && wsum->bp_data)
                            backproject(m, ic, A, cur, Fimg.data(), Fweight.data(), wsum->bp_data, wsum->bp_weight);
                    }
                }
        // power beyond the current size (:9010-9017)
        for (long ires = cur / 2 + 1; ires < m.ori_size / 2 + 1; ++ires) {
            thr_sigma2[ires] += P.power_img[ires];
            norm_corr += P.power_img[ires];
        }
        double normcorr = P.norm_correction;
        if (m.do_norm_correction) {
            double old_nc = P.norm_correction / m.avg_norm_correction;
            normcorr = old_nc * std::sqrt(norm_corr * 2.);
        }
        if (m.do_scale_correction) {
            XA /= P.scale;
            AA /= P.scale * P.scale;
        }
        double logsigma2 = 0.;
        for (long k = 0; k < npix; ++k) {
            int ires = Mres_f[k];
            int irm = r_round(1.0 * ires);
            if (ires > 0 && irm < m.sigma2_len) logsigma2 += 1 * std::log(2. * kPI * m.sigma2_noise[irm]);
        }
        double dLL = std::log(sum_weight) - min_diff2 - logsigma2;
        res[ip].dLL = dLL;
        res[ip].norm = normcorr;
        res[ip].nr_sign = (double)nr_sign;
        if (wsum) {
            for (long i = 0; i < nhalf; ++i) wsum->sigma2_noise[i] += thr_sigma2[i];
            wsum->sumw_group += sumw_group;
            if (m.do_scale_correction) {
                wsum->wsum_signal_product += XA;
                wsum->wsum_reference_power += AA;
            }
            for (long ic = 0; ic < K; ++ic) wsum->pdf_class[ic] += thr_pdf_class[ic];
            for (long i = 0; i < K * ND; ++i) wsum->pdf_direction[i] += thr_pdf_dir[i];
            wsum->sigma2_offset += sigma2_off;
            if (is2d && wsum->prior_offset_class)
                for (long i = 0; i < 2 * K; ++i) wsum->prior_offset_class[i] += thr_prior_off[i];
            if (m.do_norm_correction) wsum->avg_norm_correction += normcorr;
            wsum->LL += dLL;
            wsum->ave_Pmax += res[ip].pmax;
        }
        (void)X;
    }
    return 0;
}


// ---------------------------------------------------------------------------
// Image preparation: MlOptimiser::getFourierTransformsAndCtfs
// (src/ml_optimiser.cpp:5840-6753) for 2D single-particle images, without
// helical / multi-body / tomography branches, with --zero_mask (background
// average outside the mask), no CTF padding, no MTF or aberration
// corrections.  FFTs in double: an iterative radix-2 transform for
// power-of-two sizes, a direct DFT otherwise.
// ---------------------------------------------------------------------------
static void fft1d(std::vector<Cplx> &a, bool inverse) {
    const size_t n = a.size();
    if (n && (n & (n - 1)) == 0) {
        for (size_t i = 1, j = 0; i < n; ++i) {
            size_t bit = n >> 1;
            for (; j & bit; bit >>= 1) j ^= bit;
            j ^= bit;
            if (i < j) std::swap(a[i], a[j]);
        }
        for (size_t len = 2; len <= n; len <<= 1) {
            const double ang = 2 * kPI / (double)len * (inverse ? 1 : -1);
            for (size_t i = 0; i < n; i += len)
                for (size_t k = 0; k < len / 2; ++k) {
                    const double c = std::cos(ang * k), sn = std::sin(ang * k);
                    Cplx u = a[i + k], v = a[i + k + len / 2];
                    Cplx t{v.re * c - v.im * sn, v.re * sn + v.im * c};
                    a[i + k] = Cplx{u.re + t.re, u.im + t.im};
                    a[i + k + len / 2] = Cplx{u.re - t.re, u.im - t.im};
                }
        }
        return;
    }
    std::vector<Cplx> out(n, Cplx{0, 0});
    for (size_t k = 0; k < n; ++k)
        for (size_t x = 0; x < n; ++x) {
            const double ang = 2 * kPI * (double)((k * x) % n) / (double)n * (inverse ? 1 : -1);
            out[k].re += a[x].re * std::cos(ang) - a[x].im * std::sin(ang);
            out[k].im += a[x].re * std::sin(ang) + a[x].im * std::cos(ang);
        }
    a = out;
}

// FourierTransformer::FourierTransform of an N x N real image: FFTW half
// layout [N][N/2+1], forward transform divided by N^2 (src/fftw.cpp:335-360).
static std::vector<Cplx> rfft2_half(const std::vector<double> &img, long N) {
    const long X = N / 2 + 1;
    std::vector<Cplx> rows((size_t)N * X);
    std::vector<Cplx> line(N);
    for (long y = 0; y < N; ++y) {
        for (long x = 0; x < N; ++x) line[x] = Cplx{img[(size_t)y * N + x], 0.};
        fft1d(line, false);
        for (long x = 0; x < X; ++x) rows[(size_t)y * X + x] = line[x];
    }
    for (long x = 0; x < X; ++x) {
        for (long y = 0; y < N; ++y) line[y] = rows[(size_t)y * X + x];
        fft1d(line, false);
        for (long y = 0; y < N; ++y) {
            rows[(size_t)y * X + x].re = line[y].re / ((double)N * N);
            rows[(size_t)y * X + x].im = line[y].im / ((double)N * N);
        }
    }
    return rows;
}

// CenterFFTbySign (src/fftw.h:390-403) on a [s][s/2+1] half transform
static void center_by_sign(std::vector<Cplx> &F, long s) {
    const long X = s / 2 + 1;
    for (long i = 0; i < s; ++i)
        for (long j = 0; j < X; ++j)
            if ((i ^ j) & 1) {
                F[(size_t)i * X + j].re = -F[(size_t)i * X + j].re;
                F[(size_t)i * X + j].im = -F[(size_t)i * X + j].im;
            }
}

int oracle_prepare_images(const oracle_prep_params *pp, int64_t n, const double *images,
                          const oracle_image_meta *meta, double *fimg, double *fimg_nomask, double *fctf,
                          double *power, double *highres_Xi2, double *old_offset_rounded) {
    const long N = pp->ori_size, cur = pp->current_size, X = cur / 2 + 1, half = N / 2 + 1;
    if (N <= 0 || cur <= 0 || cur > N || (N & 1) || (cur & 1)) return -1;
    const long h = N / 2;  // Xmipp origin of an even N x N image: logical = index - N/2
    for (long p = 0; p < n; ++p) {
        const oracle_image_meta &mt = meta[p];
        const double *in = images + (size_t)p * N * N;
        std::vector<double> img((size_t)N * N, 0.);
        // norm correction (:6200-6212)
        const double f = pp->do_norm_correction ? pp->avg_norm_correction / mt.norm_correction : 1.;
        // rounded old offset (:6054), integer selfTranslate without wrap (:6214-6219;
        // src/transformations.h translate: V2(r) = V1(r - v), outside 0)
        const int dx = r_round(mt.old_offset[0]), dy = r_round(mt.old_offset[1]);
        old_offset_rounded[2 * p] = dx;
        old_offset_rounded[2 * p + 1] = dy;
        for (long y = 0; y < N; ++y)
            for (long x = 0; x < N; ++x) {
                const long sy = y - dy, sx = x - dx;
                if (sy >= 0 && sy < N && sx >= 0 && sx < N) img[(size_t)y * N + x] = f * in[(size_t)sy * N + sx];
            }
        // unmasked Fourier image (:6233-6240)
        std::vector<Cplx> Fa = rfft2_half(img, N);
        std::vector<Cplx> Fw = window_ft(Fa.data(), N, cur);
        center_by_sign(Fw, cur);
        std::memcpy(fimg_nomask + (size_t)p * cur * X * 2, Fw.data(), sizeof(Cplx) * cur * X);
        // soft mask with the average background (softMaskOutsideMap, src/mask.cpp:43-96)
        const double radius = pp->mask_radius_px, radius_p = radius + pp->width_mask_edge;
        double sum = 0., sum_bg = 0.;
        for (long y = 0; y < N; ++y)
            for (long x = 0; x < N; ++x) {
                const double r = std::sqrt((double)((y - h) * (y - h) + (x - h) * (x - h)));
                if (r < radius) continue;
                if (r > radius_p) {
                    sum += 1.;
                    sum_bg += img[(size_t)y * N + x];
                } else {
                    const double rc = 0.5 + 0.5 * std::cos(kPI * (radius_p - r) / pp->width_mask_edge);
                    sum += rc;
                    sum_bg += rc * img[(size_t)y * N + x];
                }
            }
        sum_bg /= sum;
        for (long y = 0; y < N; ++y)
            for (long x = 0; x < N; ++x) {
                const double r = std::sqrt((double)((y - h) * (y - h) + (x - h) * (x - h)));
                if (r < radius) continue;
                double &v = img[(size_t)y * N + x];
                if (r > radius_p) {
                    v = sum_bg;
                } else {
                    const double rc = 0.5 + 0.5 * std::cos(kPI * (radius_p - r) / pp->width_mask_edge);
                    v = (1 - rc) * v + rc * sum_bg;
                }
            }
        // masked Fourier image, power spectrum and high-resolution power (:6320-6350)
        Fa = rfft2_half(img, N);
        double *pw = power + (size_t)p * half;
        for (long i = 0; i < half; ++i) pw[i] = 0.;
        double xi2 = 0.;
        if (cur < N) {
            for (long i = 0; i < N; ++i) {
                const long ip = (i < half) ? i : i - N;
                for (long j = 0; j < half; ++j) {
                    const int ires = r_round(std::sqrt((double)(ip * ip + j * j)));
                    if (ires > 0 && ires < half && !(j == 0 && ip < 0)) {
                        const Cplx c = Fa[(size_t)i * half + j];
                        const double nf = c.re * c.re + c.im * c.im;
                        pw[ires] += nf;
                        if (ires >= cur / 2 + 1) xi2 += nf;
                    }
                }
            }
        }
        highres_Xi2[p] = xi2;
        Fw = window_ft(Fa.data(), N, cur);
        center_by_sign(Fw, cur);
        std::memcpy(fimg + (size_t)p * cur * X * 2, Fw.data(), sizeof(Cplx) * cur * X);
        // CTF image (CTF::getFftwImage, src/ctf.cpp:314-450: no padding,
        // frequencies of the full box, FFTW half layout of the current size)
        double *fc = fctf + (size_t)p * cur * X;
        const double xs = (double)N * pp->pixel_size;
        for (long i = 0; i < cur; ++i) {
            const long ip = (i < X) ? i : i - cur;
            for (long j = 0; j < X; ++j)
                fc[(size_t)i * X + j] = oracle_ctf(mt.defU, mt.defV, mt.defAngle, pp->kV, pp->Cs, pp->Q0, mt.Bfac,
                                                   mt.scale, mt.phase_shift, (double)j / xs, (double)ip / xs);
        }
    }
    return 0;
}

}  // extern "C"
