/*
 * relion_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * C ABI of the CPU double-precision restatement of relion_refine's CPU
 * expectation step (relion_refine without --gpu, RFLOAT = double).  Only
 * tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
 * arm may load the library built from relion_oracle.cpp; the product path
 * (libgbrelion) never links or calls it.
 *
 * Parity pins (the reference's own code, built from its sources by
 * oracle/build_ref.sh into oracle/_ref, and golden vectors of it under
 * tests/golden):
 *   - CTF value: reference tests/ctf.cpp:8-9 (getCTF(10,10) = 0.59154).
 *   - HEALPix NEST enumeration: bit-for-bit against
 *     src/Healpix_2.15a/healpix_base.cc.
 *   - The E-step itself: MlOptimiser::getAllSquaredDifferences,
 *     convertAllSquaredDifferencesToWeights and storeWeightedSums of the
 *     reference (oracle/_ref/ref_estep) on the same prepared particles give
 *     the same coarse and fine diff2, weights, significance sets, fine pose
 *     sets, best poses, PMAX, dLL, weighted sums and backprojected volumes
 *     (bit-identical on x86-64 with this build's flags).
 *   - Building blocks: Projector::project, BackProjector::backproject2Dto3D,
 *     CTF::getFftwImage, HealpixSampling, shiftImageInFourierTransform,
 *     Euler_angles2matrix, BackProjector::reconstruct and
 *     Projector::computeFourierTransformMap (oracle/_ref/ref_pin).
 */
#ifndef RELION_ORACLE_H
#define RELION_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Model and sampling state read by the E-step (MlOptimiser / MlModel /
 * HealpixSampling members).  All lengths in pixels unless stated. */
/* Host threads of the oracle's OpenMP loops; returns the number in effect. */
int oracle_set_threads(int n);

typedef struct {
    int64_t ori_size;            /* mymodel.ori_size                               */
    int64_t nr_classes;          /* mymodel.nr_classes                             */
    int64_t current_size;        /* image_current_size[optics_group]              */
    int64_t coarse_size;         /* image_coarse_size[optics_group]               */
    int64_t padding_factor;      /* PPref/BPref padding factor (2)                 */
    /* padded Fourier reference (Projector::data), one per class               */
    int64_t proj_r_max, proj_xdim, proj_ydim, proj_zdim, proj_yinit, proj_zinit;
    /* backprojector volumes (BackProjector::data / weight), one per class      */
    int64_t bp_r_max, bp_xdim, bp_ydim, bp_zdim, bp_yinit, bp_zinit;
    /* sampling (HealpixSampling)                                               */
    int64_t healpix_order;
    int64_t adaptive_oversampling;
    int64_t maximum_significants;  /* --maxsig (<=0: off)                         */
    int64_t sigma2_len;            /* XSIZE(mymodel.sigma2_noise[optics_group])   */
    int64_t do_scale_correction;
    int64_t do_norm_correction;
    int64_t do_map;
    int64_t ref_dim;             /* mymodel.ref_dim: 3 (or 0) 3D, 2 = 2D classes  */
    double pixel_size;           /* mymodel.pixel_size == particle pixel size     */
    double psi_step;             /* degrees (<=0: 360/(6*2^order))                */
    double offset_range;         /* Angstrom (command line px * pixel size)       */
    double offset_step;          /* Angstrom                                      */
    double adaptive_fraction;
    double sigma2_fudge;
    double sigma2_offset;        /* Angstrom^2                                     */
    double avg_norm_correction;
    const double *ppref;         /* [K][z][y][x][2]                                */
    const double *sigma2_noise;  /* [sigma2_len]                                    */
    const double *pdf_class;     /* [K]                                            */
    const double *pdf_direction; /* [K][ndir]                                      */
    const double *data_vs_prior; /* [K][ori/2+1] (scale correction only)           */
    const double *prior_offset_class; /* [K][2] 2D: mymodel.prior_offset_class (or NULL) */
} oracle_model;

typedef struct {
    const double *fimg;          /* [cur][cur/2+1][2] masked image FT              */
    const double *fimg_nomask;   /* [cur][cur/2+1][2]                              */
    const double *fctf;          /* [cur][cur/2+1]                                 */
    const double *power_img;     /* [ori/2+1]                                       */
    double old_offset[2];        /* pixels                                         */
    double prior[2];             /* pixels                                         */
    double highres_Xi2;
    double norm_correction;      /* metadata NORM                                   */
    double scale;                /* scale_correction[group]                         */
    double pad_;
} oracle_particle;

/* per-particle results (metadata columns written by storeWeightedSums) */
typedef struct {
    double rot, tilt, psi, xoff, yoff;
    double cls;                  /* 1-based class                                   */
    double pmax, dLL, norm;
    double nr_sign;
    double coarse_min_diff2, coarse_sum_weight, coarse_significant_weight;
    double fine_min_diff2, fine_sum_weight, fine_significant_weight;
    int64_t best_ihidden_over;   /* fine-pass index of the PMAX pose               */
    int64_t pad_;
} oracle_result;

/* optional per-particle debug arrays (NULL to skip) */
typedef struct {
    double *coarse_diff2;        /* [R*T] before conversion, -999 = not computed   */
    double *coarse_weight;       /* [R*T] after conversion                          */
    uint8_t *coarse_significant; /* [R*T]                                          */
    double *fine_diff2;          /* [R*T*nOR*nOT]                                   */
    double *fine_weight;         /* [R*T*nOR*nOT]                                   */
} oracle_debug;

/* weighted sums (MlWsumModel members), accumulated (+=) by the oracle */
typedef struct {
    double *sigma2_noise;        /* [ori/2+1]                                       */
    double *pdf_class;           /* [K]                                             */
    double *pdf_direction;       /* [K][ndir]                                       */
    double *bp_data;             /* [K][bz][by][bx][2]                              */
    double *bp_weight;           /* [K][bz][by][bx]                                 */
    double sigma2_offset, sumw_group, LL, ave_Pmax, avg_norm_correction;
    double wsum_signal_product, wsum_reference_power;
    double pad_;
    double *prior_offset_class;  /* [K][2] 2D: += weight * pixel * (old offset + shift) */
} oracle_wsum;

int oracle_expectation(const oracle_model *m, int64_t n, const oracle_particle *parts,
                       oracle_result *res, oracle_debug *dbg, oracle_wsum *wsum);

/* --- image preparation (MlOptimiser::getFourierTransformsAndCtfs) -------- */
typedef struct {
    int64_t ori_size;            /* image_full_size                                 */
    int64_t current_size;        /* image_current_size                              */
    int64_t do_norm_correction;
    int64_t pad_;
    double pixel_size;
    double mask_radius_px;       /* particle_diameter / (2 pixel)                   */
    double width_mask_edge;      /* --width_mask_edge (pixels)                      */
    double avg_norm_correction;
    double kV, Cs, Q0;           /* optics group: voltage, spherical aberration, amplitude contrast */
} oracle_prep_params;

typedef struct {
    double old_offset[2];        /* pixels, before rounding                         */
    double norm_correction;
    double defU, defV, defAngle; /* Angstrom, Angstrom, degrees                     */
    double Bfac, scale, phase_shift;
} oracle_image_meta;

/* Real-space particle images [n][ori][ori] (row y, column x) -> the E-step
 * inputs: masked and unmasked Fourier images [n][cur][cur/2+1][2], CTF
 * images [n][cur][cur/2+1], power spectra [n][ori/2+1], highres_Xi2 [n] and
 * the rounded old offsets [n][2]. */
int oracle_prepare_images(const oracle_prep_params *pp, int64_t n, const double *images,
                          const oracle_image_meta *meta, double *fimg, double *fimg_nomask, double *fctf,
                          double *power, double *highres_Xi2, double *old_offset_rounded);

/* --- reconstruction side (oracle_mstep.cpp) ----------------------------- */
typedef struct {
    int64_t ori_size, ref_dim, pad; /* integer padding factor                          */
    int64_t r_max;                  /* BackProjector r_max                              */
    int64_t xdim, ydim, zdim, yinit, zinit; /* data / weight layout (x from 0)          */
} oracle_bp_geom;

typedef struct {
    int64_t max_iter_preweight;  /* --gridding_iter                                    */
    int64_t do_map;
    int64_t skip_gridding;       /* default of relion_refine: no --dont_skip_gridding  */
    int64_t minres_map;
    double tau2_fudge;
    double normalise;            /* wsum pdf_class of the class                        */
} oracle_recon_params;

/* data: complex [zdim][ydim][xdim][2], weight [zdim][ydim][xdim]; modified in place */
int oracle_bp_symmetrise(const oracle_bp_geom *g, double *data, double *weight);
/* all shell arrays [ori/2+1]; tau2_io read and written */
int oracle_update_ssnr(const oracle_bp_geom *g, const double *weight, double tau2_fudge, double *tau2_io,
                       double *sigma2_out, double *dvp_out, double *cov_out, const double *fsc,
                       int64_t update_tau2_with_fsc, int64_t is_whole_instead_of_half);
/* real-space map [ori]^ref_dim (z, y, x) */
int oracle_reconstruct(const oracle_bp_geom *g, const double *data, const double *weight,
                       const oracle_recon_params *p, const double *tau2, double *vol_out);
/* map [ori]^ref_dim -> padded Fourier reference (projector layout of current_size) and power [ori/2+1] */
int oracle_projector_from_map(int64_t ori, int64_t ref_dim, int64_t padding_factor, const double *vol,
                              int64_t current_size, int64_t do_gridding, int64_t min_ires, double *proj_out,
                              double *power_out);
/* Fourier shell correlation of two maps [ori]^ref_dim -> fsc [ori/2+1] */
int oracle_fsc(int64_t ori, int64_t ref_dim, const double *m1, const double *m2, double *fsc);

/* --- building blocks exposed for unit checks --------------------------- */
double oracle_ctf(double defU, double defV, double defAng, double kV, double Cs,
                  double Q0, double Bfac, double scale, double phase_shift,
                  double X, double Y);
/* number of coarse directions/psi/translations */
int oracle_sampling_sizes(int64_t order, double psi_step, double offset_range,
                          double offset_step, int64_t *ndir, int64_t *npsi, int64_t *ntrans);
/* coarse direction table: rot/tilt (degrees) and NEST pixel per direction */
int oracle_directions(int64_t order, double *rot, double *tilt, int64_t *ipix);
/* oversampled orientations of (idir, ipsi): nOR entries */
int oracle_oversampled_orientations(int64_t order, double psi_step, int64_t idir, int64_t ipsi,
                                    int64_t ov, double *rot, double *tilt, double *psi);
/* translations (Angstrom) of the coarse grid */
int oracle_translations(double offset_range, double offset_step, double *tx, double *ty);
/* oversampled translations of itrans, in pixels */
int oracle_oversampled_translations(double offset_range, double offset_step, int64_t itrans,
                                    int64_t ov, double pixel_size, double *tx, double *ty);
/* HEALPix raw functions */
void oracle_hpx_pix2ang_z_phi(int64_t order, int64_t pix, double *z, double *phi);
void oracle_hpx_nest2xyf(int64_t order, int64_t pix, int64_t *ix, int64_t *iy, int64_t *face);
int64_t oracle_hpx_xyf2nest(int64_t order, int64_t ix, int64_t iy, int64_t face);
/* Euler (rot,tilt,psi) -> 3x3 row-major */
void oracle_euler(double rot, double tilt, double psi, double *A);
/* Building blocks, for checks against the reference's own code: the
 * projection of class iclass of m->ppref at the Euler matrix A (row-major)
 * into a [size][size/2+1] complex image; the backprojection of such an
 * image with weights Mw into volumes of the m->bp_* geometry (added to
 * bp_data complex / bp_weight); the phase shift of an image by (x, y)
 * pixels of a box of oridim. */
void oracle_project(const oracle_model *m, int64_t iclass, const double *A, int64_t size, double *out);
void oracle_backproject(const oracle_model *m, int64_t iclass, const double *A, int64_t size, const double *f2d,
                        const double *Mw, double *bp_data, double *bp_weight);
void oracle_shift_ft(const double *in, int64_t size, double oridim, double xshift, double yshift, double *out);

#ifdef __cplusplus
}
#endif
#endif
