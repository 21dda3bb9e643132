// sampling.h -- pose grid of the E-step (host side of libgbrelion).
//
// HEALPix NEST directions, in-plane (psi) angles, the 2D translation grid and
// their adaptive oversampling, following the reference's HealpixSampling
// (src/healpix_sampling.cpp) and Healpix_Base (src/Healpix_2.15a/
// healpix_base.cc).  The enumeration order and the hidden-variable packing
// are the reference's, because the significance masks and the per-particle
// metadata are indexed by them:
//   coarse  ihidden      = ((iclass*ndir + idir)*npsi + ipsi)*ntrans + itrans
//   fine    ihidden_over = ihidden*nOR*nOT + iover_rot*nOT + iover_trans
// (src/healpix_sampling.cpp:1704-1722).  Double-precision expressions are
// evaluated in the reference's order; this file is compiled with
// -ffp-contract=off so the angles come out bit-identical.
#pragma once
#include <cmath>
#include <vector>

namespace gbr {

constexpr double kPi = 3.14159265358979323846;
constexpr double kHalfPiHpx = 1.570796326794896619231321691639751442099;

inline int iround(double x) { return (x > 0) ? (int)(x + 0.5) : (int)(x - 0.5); }
inline int iceil(double x) { return (x == (int)x) ? (int)x : ((x > 0) ? (int)(x + 1) : (int)x); }

// One HEALPix resolution in the NEST scheme.
class HealpixNest {
  public:
    explicit HealpixNest(int order)
        : order_(order), nside_(1 << order), npface_((1 << order) << order), npix_(12 * npface_) {
        fact2_ = 4. / npix_;
        fact1_ = (nside_ << 1) * fact2_;
    }
    int npix() const { return npix_; }
    int nside() const { return nside_; }

    void pix_to_xyf(int pix, int &ix, int &iy, int &face) const {
        face = pix >> (2 * order_);
        int p = pix & (npface_ - 1);
        ix = compact_even_bits(p);
        iy = compact_even_bits(p >> 1);
    }
    int xyf_to_pix(int ix, int iy, int face) const {
        return (face << (2 * order_)) + (spread_bits(ix) | (spread_bits(iy) << 1));
    }
    // z = cos(theta) and phi of the pixel centre.
    void pix_to_z_phi(int pix, double &z, double &phi) const {
        static const int ring_of_face[12] = {2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4};
        static const int phi_of_face[12] = {1, 3, 5, 7, 0, 2, 4, 6, 1, 3, 5, 7};
        int face, ix, iy;
        pix_to_xyf(pix, ix, iy, face);
        const int nl4 = 4 * nside_;
        const int jr = (ring_of_face[face] << order_) - ix - iy - 1;
        int nr, kshift;
        if (jr < nside_) {
            nr = jr;
            z = 1 - nr * nr * fact2_;
            kshift = 0;
        } else if (jr > 3 * nside_) {
            nr = nl4 - jr;
            z = nr * nr * fact2_ - 1;
            kshift = 0;
        } else {
            nr = nside_;
            z = (2 * nside_ - jr) * fact1_;
            kshift = (jr - nside_) & 1;
        }
        int jp = (phi_of_face[face] * nr + ix - iy + 1 + kshift) / 2;
        if (jp > nl4) jp -= nl4;
        if (jp < 1) jp += nl4;
        phi = (jp - (kshift + 1) * 0.5) * (kHalfPiHpx / nr);
    }

  private:
    static int compact_even_bits(int v) {
        int r = 0;
        for (int b = 0; b < 15; ++b) r |= ((v >> (2 * b)) & 1) << b;
        return r;
    }
    static int spread_bits(int v) {
        int r = 0;
        for (int b = 0; b < 15; ++b) r |= ((v >> b) & 1) << (2 * b);
        return r;
    }
    int order_, nside_, npface_, npix_;
    double fact1_, fact2_;
};

// rot in [-180,180], tilt in [0,180] (HealpixSampling::checkDirection).
inline void wrap_direction(double &rot, double &tilt) {
    if (tilt < 0.) {
        tilt = -tilt;
        rot += 180.;
    }
    while (rot > 180. || rot < -180.) rot += (rot > 180.) ? -360. : 360.;
}

inline void healpix_angles(const HealpixNest &h, int pix, double &rot, double &tilt) {
    double z, phi;
    h.pix_to_z_phi(pix, z, phi);
    rot = phi * 180 / kPi;
    tilt = acos(z) * 180. / kPi;
    wrap_direction(rot, tilt);
}

// Euler angles (degrees, ZYZ as in src/euler.cpp:52-91) -> rotation matrix A
// (row-major).  Projection uses A^-1 = A^T.
inline void euler_to_matrix(double rot, double tilt, double psi, double A[9]) {
    const double a = rot * kPi / 180, b = tilt * kPi / 180, g = psi * kPi / 180;
    const double ca = cos(a), cb = cos(b), cg = cos(g), sa = sin(a), sb = sin(b), sg = sin(g);
    const double cc = cb * ca, cs = cb * sa, sc = sb * ca, ss = sb * sa;
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

struct PoseGrid {
    bool is3d = true;  // false: 2D classification (in-plane psi only)
    int order = 0, oversampling = 0;
    double psi_step = 0, offset_range = 0, offset_step = 0;  // degrees, Angstrom
    std::vector<double> dir_rot, dir_tilt;
    std::vector<int> dir_pix;
    std::vector<double> psi;
    std::vector<double> trans_x, trans_y;  // Angstrom

    long ndir() const { return (long)dir_rot.size(); }
    long npsi() const { return (long)psi.size(); }
    long ntrans() const { return (long)trans_x.size(); }
    int nover_rot() const { return iround(std::pow(2., oversampling * (is3d ? 3 : 1))); }
    int nover_trans() const { return iround(std::pow(2., oversampling * 2)); }

    // HealpixSampling::initialise / setOrientations / setTranslations
    // (src/healpix_sampling.cpp:55-120, 477-560, 291-440): in 3D every HEALPix
    // pixel (C1) x psi; in 2D one direction (rot = tilt = 0) x psi, psi step 10
    // degrees by default.
    void build(int order_, double psi_step_in, double range, double step, int ov, bool three_d = true) {
        is3d = three_d;
        order = order_;
        oversampling = ov;
        dir_rot.clear(); dir_tilt.clear(); dir_pix.clear(); psi.clear(); trans_x.clear(); trans_y.clear();
        if (is3d) {
            const HealpixNest h(order);
            for (int p = 0; p < h.npix(); ++p) {  // C1: every pixel is kept
                double r, t;
                healpix_angles(h, p, r, t);
                dir_rot.push_back(r);
                dir_tilt.push_back(t);
                dir_pix.push_back(p);
            }
        } else {
            dir_rot.push_back(0.);
            dir_tilt.push_back(0.);
            dir_pix.push_back(-1);
        }
        double ps = psi_step_in > 0 ? psi_step_in
                                    : (is3d ? 360. / (6 * iround(std::pow(2., order))) : 10.);
        const int nr_psi = iceil(360. / ps);
        psi_step = 360. / (double)nr_psi;
        for (int i = 0; i < nr_psi; ++i) psi.push_back(i * psi_step);
        offset_range = range;
        offset_step = step;
        const int maxp = iceil(offset_range / offset_step);
        for (long ix = -maxp; ix <= maxp; ++ix)
            for (long iy = -maxp; iy <= maxp; ++iy) {
                const double xo = ix * offset_step, yo = iy * offset_step;
                if (xo * xo + yo * yo < (offset_range * offset_range) + 0.001) {
                    trans_x.push_back(xo);
                    trans_y.push_back(yo);
                }
            }
    }

    // Oversampled orientations of coarse (idir, ipsi): nover_rot() entries in
    // the reference's order (child pixel j-major, i-minor, then child psi).
    void fine_orientations(long idir, long ipsi, double *rot, double *tilt, double *ps) const {
        if (!is3d) {
            // 2D: only the in-plane angle is oversampled, wrapped to (-180, 180]
            // (pushbackOversampledPsiAngles, src/healpix_sampling.cpp:1941-1968)
            const int n = iround(std::pow(2., oversampling));
            for (int k = 0; k < n; ++k) {
                double o = psi[ipsi] - 0.5 * psi_step + (0.5 + k) * psi_step / n;
                if (o > 180.) o -= 360.;
                rot[k] = 0.;
                tilt[k] = 0.;
                ps[k] = o;
            }
            return;
        }
        const HealpixNest base(order), fine(order + oversampling);
        const int fact = fine.nside() / base.nside();
        int x, y, face;
        base.pix_to_xyf(dir_pix[idir], x, y, face);
        const int npsi_over = iround(std::pow(2., oversampling));
        int n = 0;
        for (int j = fact * y; j < fact * (y + 1); ++j)
            for (int i = fact * x; i < fact * (x + 1); ++i) {
                double r, t;
                healpix_angles(fine, fine.xyf_to_pix(i, j, face), r, t);
                for (int k = 0; k < npsi_over; ++k, ++n) {
                    rot[n] = r;
                    tilt[n] = t;
                    ps[n] = psi[ipsi] - 0.5 * psi_step + (0.5 + k) * psi_step / npsi_over;
                }
            }
    }
    // One oversampled orientation (index ior of fine_orientations) of (idir, ipsi).
    void fine_orientation(long idir, long ipsi, long ior, double &rot, double &tilt, double &ps) const {
        const int npsi_over = iround(std::pow(2., oversampling));
        const int k = (int)(ior % npsi_over);
        ps = psi[ipsi] - 0.5 * psi_step + (0.5 + k) * psi_step / npsi_over;
        if (!is3d) {
            if (ps > 180.) ps -= 360.;
            rot = 0.;
            tilt = 0.;
            return;
        }
        const HealpixNest base(order), fine(order + oversampling);
        const int fact = fine.nside() / base.nside();
        int x, y, face;
        base.pix_to_xyf(dir_pix[idir], x, y, face);
        const int c = (int)(ior / npsi_over);
        healpix_angles(fine, fine.xyf_to_pix(fact * x + c % fact, fact * y + c / fact, face), rot, tilt);
    }
    // Oversampled translations of itrans in pixels (ox-major, oy-minor).
    void fine_translations(long itrans, double pixel, double *tx, double *ty) const {
        const int n = iround(std::pow(2., oversampling));
        int m = 0;
        for (int ox = 0; ox < n; ++ox) {
            const double x = trans_x[itrans] - 0.5 * offset_step + (0.5 + ox) * offset_step / n;
            for (int oy = 0; oy < n; ++oy, ++m) {
                const double y = trans_y[itrans] - 0.5 * offset_step + (0.5 + oy) * offset_step / n;
                tx[m] = x / pixel;
                ty[m] = y / pixel;
            }
        }
    }
};

}  // namespace gbr
