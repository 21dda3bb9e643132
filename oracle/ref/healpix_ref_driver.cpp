/*
 * healpix_ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * A thin C shim over the reference's own Healpix_Base class
 * (src/Healpix_2.15a/healpix_base.{h,cc}), compiled together with those
 * reference sources by oracle/build_ref.sh into oracle/_ref/libref_healpix.so.
 * Tests compare the oracle's and the product's HEALPix bookkeeping with it.
 */
#include "src/Healpix_2.15a/healpix_base.h"

extern "C" {
void ref_hpx_pix2ang_z_phi(int order, int pix, double *z, double *phi) {
    Healpix_Base h(order, NEST);
    h.pix2ang_z_phi(pix, *z, *phi);
}
void ref_hpx_nest2xyf(int order, int pix, int *ix, int *iy, int *face) {
    Healpix_Base h(order, NEST);
    h.nest2xyf(pix, *ix, *iy, *face);
}
int ref_hpx_xyf2nest(int order, int ix, int iy, int face) {
    Healpix_Base h(order, NEST);
    return h.xyf2nest(ix, iy, face);
}
int ref_hpx_npix(int order) {
    Healpix_Base h(order, NEST);
    return h.Npix();
}
int ref_hpx_nside(int order) {
    Healpix_Base h(order, NEST);
    return h.Nside();
}
}
