/*
 * gbrelion.h -- C ABI of libgbrelion, a GB300-native (sm_103a) expectation
 * step for RELION's relion_refine.
 *
 * The reference plugs its accelerated E-step into MlOptimiser through
 * opaque handles (src/ml_optimiser.h:108-109, gpuOptimisers/accDataBundles)
 * and one dispatch function (src/ml_optimiser.cpp:78-97).  Each entry point
 * below replaces one call of that surface; the comment on each names it.
 * All entry points return 0 on success or a negative gbr_status; the text of
 * the last error of the calling thread is available from gbr_last_error().
 * No entry point takes or returns a PyTorch or C++ type.
 *
 * Threads: like the reference's threads, each with its MlOptimiserCuda on
 * one MlDeviceBundle, several threads may drive their own workers of one
 * bundle at once.  Calls that run work on the bundle's shared state (E-step,
 * image preparation, volumes, model arrays, reconstruction) hold a
 * bundle-wide lock and are serialised; one worker is used by one thread at a
 * time.
 *
 * Layout conventions (FFTW half-transform, as in the reference):
 *   a 2D Fourier image of size s is stored row-major as [s][s/2+1]; row i
 *   holds frequency y = i for i <= s/2 and y = i - s otherwise.
 *   Complex values are interleaved (re, im).
 *   A padded 3D reference / backprojector volume is [zdim][ydim][xdim] with
 *   logical origin (x=0, y=yinit, z=zinit), as Projector::data
 *   (src/projector.cpp:59-90).
 */
#ifndef GBRELION_H
#define GBRELION_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    GBR_OK = 0,
    GBR_ERR_INVALID = -1,      /* bad argument / size                       */
    GBR_ERR_CUDA = -2,         /* CUDA runtime error                        */
    GBR_ERR_OOM = -3,          /* device memory budget exceeded             */
    GBR_ERR_NUMERICAL = -4,    /* zero sum of weights / no significant pose */
    GBR_ERR_STATE = -5,        /* call out of order (e.g. no reference yet) */
    GBR_ERR_UNSUPPORTED = -6   /* option outside the implemented path       */
} gbr_status;

/* Precision of the coarse-pass cross-term contraction. */
typedef enum {
    GBR_PREC_FP32 = 0,         /* plain path: FP32 SIMT, matches the CPU oracle */
    GBR_PREC_BF16 = 1          /* precision form: tcgen05 BF16, FP32 accumulate */
} gbr_precision;

/* Model, sampling and option state of one iteration (the MlOptimiser /
 * MlModel / HealpixSampling members the E-step reads). */
typedef struct {
    int64_t ori_size;            /* mymodel.ori_size                          */
    int64_t nr_classes;          /* mymodel.nr_classes                        */
    int64_t current_size;        /* image_current_size (fine pass, wsums)     */
    int64_t coarse_size;         /* image_coarse_size (coarse pass)           */
    int64_t padding_factor;      /* projector / backprojector padding (2)     */
    int64_t healpix_order;       /* --healpix_order                          */
    int64_t adaptive_oversampling;   /* --oversampling (1)                   */
    int64_t maximum_significants;    /* --maxsig (<= 0: off)                 */
    int64_t sigma2_len;          /* XSIZE(mymodel.sigma2_noise[group])       */
    int64_t do_scale_correction; /* --scale                                  */
    int64_t do_norm_correction;  /* --norm                                   */
    int64_t do_map;              /* !--no_map                                */
    int64_t precision;           /* gbr_precision                            */
    int64_t ref_dim;             /* mymodel.ref_dim: 3 (or 0) 3D refinement /
                                    classification, 2 = 2D classification    */
    double pixel_size;           /* Angstrom per pixel                       */
    double psi_step;             /* degrees; <= 0: 360/(6*2^order)           */
    double offset_range;         /* Angstrom                                 */
    double offset_step;          /* Angstrom                                 */
    double adaptive_fraction;    /* --adaptive_fraction (0.999)              */
    double sigma2_fudge;         /* --sigma2_fudge (1)                       */
    double sigma2_offset;        /* mymodel.sigma2_offset, Angstrom^2        */
    double avg_norm_correction;  /* mymodel.avg_norm_correction              */
} gbr_model_desc;

/* One batch of particles (one image each, one optics group).  Pointers are
 * host memory unless `device_resident` is set, in which case they are device
 * pointers on the bundle's GPU.  Sizes: cur = current_size, X = cur/2+1. */
typedef struct {
    int64_t n;                   /* number of particles                      */
    int64_t device_resident;     /* 0: host pointers (copied in), 1: device   */
    const float *fimg;           /* [n][cur][X][2] masked image FT            */
    const float *fimg_nomask;    /* [n][cur][X][2] unmasked image FT          */
    const float *fctf;           /* [n][cur][X]    CTF image                   */
    const double *power_img;     /* [n][ori/2+1]   power spectrum             */
    const double *old_offset;    /* [n][2] pixels                             */
    const double *prior;         /* [n][2] pixels                             */
    const double *highres_Xi2;   /* [n]                                       */
    const double *norm_correction; /* [n] metadata NORM                       */
    const double *scale;         /* [n] scale_correction of the group         */
} gbr_particle_batch;

/* Per-particle metadata written back by the E-step (the exp_metadata columns
 * set in storeWeightedSums, src/ml_optimiser.cpp:8810-8870, :9040-9060). */
typedef struct {
    double rot, tilt, psi;       /* degrees, best (PMAX) pose                */
    double xoff, yoff;           /* pixels                                   */
    double cls;                  /* 1-based class                            */
    double pmax;                 /* max normalised weight                    */
    double dLL;                  /* log-likelihood contribution              */
    double norm;                 /* norm correction                          */
    double nr_sign;              /* significant coarse samples               */
    double coarse_min_diff2, coarse_sum_weight, coarse_significant_weight;
    double fine_min_diff2, fine_sum_weight, fine_significant_weight;
    int64_t best_ihidden_over;   /* fine-pass hidden index of the PMAX pose  */
    int64_t n_fine;              /* fine poses evaluated                     */
} gbr_particle_result;

/* Scalar and per-shell weighted sums (MlWsumModel), accumulated over all
 * batches since the last gbr_bundle_reset_wsum(). */
typedef struct {
    double *sigma2_noise;        /* [ori/2+1]                                */
    double *pdf_class;           /* [K]                                      */
    double *pdf_direction;       /* [K][ndir]                                */
    double sigma2_offset, sumw_group, LL, ave_Pmax, avg_norm_correction;
    double wsum_signal_product, wsum_reference_power;
    double reserved_;
} gbr_wsum;

typedef struct gbr_bundle gbr_bundle;
typedef struct gbr_worker gbr_worker;

/* Text of the last error on this thread ("" if none).  Returns its length. */
size_t gbr_last_error(char *buf, size_t len);

/* Library / kernel build identification (e.g. "sm_103a"). */
const char *gbr_version(void);

/* new MlDeviceBundle(MlOptimiser*) + setDevice(id) + setupFixedSizedObjects()
 * (src/ml_optimiser.cpp:3579-3582, src/acc/cuda/cuda_ml_optimiser.cu:85-152).
 * Also initialises the zeroed backprojector volumes
 * (AccBackprojector::setMdlDim/initMdl) from current_size. */
int gbr_bundle_create(const gbr_model_desc *desc, int device, gbr_bundle **out);

/* AccProjector::setMdlDim(xdim,ydim,zdim,yinit,zinit,r_max,pad) + initMdl
 * (src/acc/acc_projector_impl.h:5-105): upload the padded Fourier reference
 * of one class, [zdim][ydim][xdim] complex, single precision. */
int gbr_projector_upload(gbr_bundle *b, int64_t iclass, const float *data, int64_t xdim,
                         int64_t ydim, int64_t zdim, int64_t yinit, int64_t zinit,
                         int64_t r_max, int64_t padding_factor);

/* Model arrays read by the E-step: mymodel.sigma2_noise[group] (sigma2_len),
 * pdf_class [K], pdf_direction [K][ndir], data_vs_prior_class [K][ori/2+1]
 * (may be NULL unless do_scale_correction). */
int gbr_model_set_arrays(gbr_bundle *b, const double *sigma2_noise, const double *pdf_class,
                         const double *pdf_direction, const double *data_vs_prior);

/* 2D classification (ref_dim 2): mymodel.prior_offset_class [K][2], the
 * per-class offset prior that replaces the particle's prior in pdf_offset
 * and sigma2_offset (src/ml_optimiser.cpp:7829-7833, 8449-8456).  Zero until
 * set; rejected for 3D models. */
int gbr_model_set_class_offsets(gbr_bundle *b, const double *prior_offset_class);

/* setupTunableSizedObjects(allocationSize) (cuda_ml_optimiser.cu:154-226):
 * cap the device memory the bundle and its workers may use. */
int gbr_bundle_reserve(gbr_bundle *b, size_t bytes);

/* new MlOptimiserCuda(MlOptimiser*, bundle, name) (src/ml_optimiser.cpp:3587). */
int gbr_worker_create(gbr_bundle *b, gbr_worker **out);

/* Keep host copies of the last call's intermediate arrays for
 * gbr_worker_debug_fetch (the RELION_TESTING dumps of
 * src/ml_optimiser.cpp:4600-4700 serve the same purpose).  The read-back
 * does not change the computation: the call runs the same passes, kernels
 * and sparse stores as without it, and the copies are taken per pass. */
int gbr_worker_set_debug(gbr_worker *w, int on);

/* Worker settings for tests and tuning (the reference has no counterpart;
 * its equivalents are compile-time constants).  The library reads no
 * environment variable: every setting is made through this call. */
typedef enum {
    GBR_OPT_DEBUG = 1,        /* as gbr_worker_set_debug                             */
    GBR_OPT_FINE_MODE = 2,    /* fine pass: 0 by significant density (default),
                                 1 always dense, 2 always sparse                      */
    GBR_OPT_COARSE_ROWS = 3,  /* precision form: 0 skip coarse rows far above the
                                 minimum (default), 1 read every row                  */
    GBR_OPT_CAND_CAP = 4,     /* coarse candidate-list entries per particle (65536)   */
    GBR_OPT_CAND_BUF = 5,     /* block-local candidate buffer entries (0: all)        */
    GBR_OPT_BATCH_CAP = 6,    /* particles per pass of a call (0: from the budget)    */
    GBR_OPT_TILE_GROUP = 7,   /* precision form: orientation tiles of 128 rows per
                                 group of the coarse kernel's tile order (0: 32)     */
    GBR_OPT_KEEP_A = 8,       /* precision form: 1 reads the projection tiles with
                                 an L2 keep policy (default 0)                        */
    GBR_OPT_PAIR = 9,         /* precision form: 1 runs the coarse cross term on SM
                                 pairs (tcgen05 cta_group::2; default 0)             */
    GBR_OPT_BP_FLUSH = 10,    /* particles collected in the FP32 staging volumes
                                 before they are added into the FP64 volumes
                                 (default 2048; 0: after every pass).  Reading,
                                 replacing or reconstructing the volumes flushes
                                 first.                                               */
    GBR_OPT_GRAPH = 11,       /* 1 (default): the coarse part of a pass (up to the
                                 read-back of the fine job lists) is captured as
                                 a CUDA graph on the second pass of a batch size
                                 and replayed while buffers, model and settings
                                 are unchanged; 0: always launched directly      */
    GBR_OPT_BP_DIRECT = 12    /* sparse fine pass: 1 inserts each job's weighted
                                 slices into the backprojection's staging volumes
                                 from the weighted-sum kernel (no per-orientation
                                 slice sums; pays when particles share few
                                 orientations, late iterations); 0 (default) sums
                                 slices per orientation first                    */
} gbr_worker_option;
int gbr_worker_set_option(gbr_worker *w, int option, int64_t value);

/* MlOptimiserCuda::doThreadExpectationSomeParticles(thread_id)
 * (cuda_ml_optimiser.cu:250-299 -> accDoExpectationOneParticle,
 * src/acc/acc_ml_optimiser_impl.h:3673), for a batch of particles:
 * coarse search, significance, fine search, weights, weighted sums and
 * backprojection into the bundle's volumes.  `res` has batch->n entries. */
int gbr_expect_batch(gbr_worker *w, const gbr_particle_batch *batch, gbr_particle_result *res);

/* ---- coarse pass restricted to proposed orientations ------------------
 * No counterpart in the reference: its coarse pass scores every orientation
 * (getAllSquaredDifferencesCoarse, src/acc/acc_ml_optimiser_impl.h:1016-1414;
 * CPU src/ml_optimiser.cpp:7098-7700).  Here each particle may score only a
 * set of orientation blocks, e.g. the ones a pose-proposal network puts its
 * mass on, with the exhaustive search kept for particles whose list starts
 * with GBR_ALL_BLOCKS.  A block is one parent HEALPix pixel: the four sibling
 * directions 4 j .. 4 j + 3 of the coarse NEST grid (of class
 * block / (ndir / 4)), with every psi angle and every translation.  Poses in
 * blocks a particle does not score get weight zero; significance, the fine
 * pass, the weighted sums and the backprojection then run as in
 * gbr_expect_batch.  Precision form only (tcgen05), 3D grids with
 * 4 x npsi a multiple of 32 and at most 256, at most 128 translations;
 * GBR_ERR_UNSUPPORTED otherwise. */
#define GBR_ALL_BLOCKS (-2)

/* Number of orientation blocks (K x ndir / 4), directions per block (4) and
 * projection-table rows per block (4 npsi). */
int gbr_orientation_blocks(const gbr_bundle *b, int64_t *nblocks, int64_t *dirs_per_block, int64_t *rows_per_block);

/* gbr_expect_batch with the coarse pass restricted per particle: blocks is
 * host int32 [batch->n][m]; row i lists the blocks particle i scores
 * (negative entries are ignored, repeats scored once), or starts with
 * GBR_ALL_BLOCKS for the exhaustive search. */
int gbr_expect_batch_blocks(gbr_worker *w, const gbr_particle_batch *batch, const int32_t *blocks, int64_t m,
                            gbr_particle_result *res);

/* ---- image preparation (the step before the search) ------------------- */

/* Optics and masking of MlOptimiser::getFourierTransformsAndCtfs. */
typedef struct {
    double kV;                   /* optics group voltage (kV)                  */
    double Cs;                   /* spherical aberration (mm)                  */
    double Q0;                   /* amplitude contrast                         */
    double particle_diameter;    /* --particle_diameter (Angstrom): the mask
                                    radius is diameter / (2 pixel size)        */
    double width_mask_edge;      /* --width_mask_edge (pixels, default 5)      */
    double reserved_;
} gbr_optics_desc;

/* A batch of real-space particle images (2D, ori_size x ori_size). */
typedef struct {
    int64_t n;
    int64_t device_resident;     /* 0: host arrays (copied in), 1: device      */
    const float *images;         /* [n][ori][ori], row y, column x             */
    const double *old_offset;    /* [n][2] pixels (rounded by the library, as
                                    the reference does before shifting)        */
    const double *prior;         /* [n][2] pixels                              */
    const double *norm_correction;  /* [n] metadata NORM                       */
    const double *scale;         /* [n] scale correction of the group          */
    const double *ctf;           /* [n][6] defocusU, defocusV (Angstrom),
                                    defocus angle (degrees), B-factor,
                                    CTF scale, phase shift (degrees)           */
} gbr_image_batch;

/* Set the optics / mask parameters used by the two calls below. */
int gbr_bundle_set_optics(gbr_bundle *b, const gbr_optics_desc *optics);

/* MlOptimiser::getFourierTransformsAndCtfs (src/ml_optimiser.cpp:5840-6753;
 * GPU variant src/acc/acc_ml_optimiser_impl.h:11-1013) for a batch, with
 * --zero_mask semantics (average background outside the soft mask), no CTF
 * padding and no MTF / aberration terms: norm correction, integer shift by
 * the rounded old offset, FFT of the unmasked and masked image, window to
 * the current size, power spectrum, high-resolution power and CTF image.
 * Outputs are DEVICE arrays in gbr_particle_batch layout: fimg, fimg_nomask
 * complex [n][cur][cur/2+1], fctf [n][cur][cur/2+1], power_img [n][ori/2+1],
 * highres_Xi2 [n], old_offset_rounded [n][2]. */
int gbr_prepare_images(gbr_worker *w, const gbr_image_batch *in, void *fimg, void *fimg_nomask, float *fctf,
                       double *power_img, double *highres_Xi2, double *old_offset_rounded);

/* gbr_prepare_images followed by gbr_expect_batch on its outputs: the E-step
 * of a batch of raw images (the reference's per-particle image preparation
 * plus accDoExpectationOneParticle). */
int gbr_expect_images(gbr_worker *w, const gbr_image_batch *in, gbr_particle_result *res);

/* Stage a host image batch (page-locked memory, for the copy to run
 * asynchronously) into the next of the worker's two device slots.  The copy
 * runs on a copy stream of the worker's own; it is issued by the next
 * gbr_expect_images once that call has queued its own small input copies
 * (the host-to-device copy engine serves copies in the order they were
 * queued, across streams), so it uploads during that call's E-step.  A later
 * gbr_expect_images with the same batch (same images pointer and count)
 * prepares it from the slot instead of copying it then.  Staging batch i + 1
 * before gbr_expect_images(batch i) overlaps its upload with batch i's
 * compute (the pinned-memory reader feeding the batch queue).  The caller
 * keeps the host batch unchanged until it is used. */
int gbr_stage_images(gbr_worker *w, const gbr_image_batch *in);

/* ---- data formats (MRC image stacks, STAR metadata) --------------------- */

/* MRC header fields (src/rwMRC.h): sizes, data mode, extended-header bytes,
 * byte order, pixel size (cell a / mx) and the offset of the first image. */
typedef struct {
    int64_t nx, ny, nz, mode, nsymbt, swapped;
    double pixel_size;
    int64_t data_offset;
} gbr_mrc_header;

int gbr_mrc_read_header(const char *path, gbr_mrc_header *out);
/* Images [first, first + count) of a stack as float32 [count][ny][nx] into
 * `out` (page-locked memory for a direct device upload), `nthreads` readers
 * (Image::read through readMRC, src/rwMRC.h:140-240; modes 0, 1, 2, 6, 12,
 * 101). */
int gbr_mrc_read_images(const char *path, int64_t first, int64_t count, float *out, int nthreads);
/* A float32 (mode 2) stack [nz][ny][nx] with the given pixel size. */
int gbr_mrc_write_stack(const char *path, const float *data, int64_t nx, int64_t ny, int64_t nz,
                        double pixel_size);

/* STAR files (MetaDataTable::read, src/metadata_table.cpp): data_ blocks with
 * a loop_ table or label / value pairs. */
typedef struct gbr_star gbr_star;
int gbr_star_read(const char *path, gbr_star **out);
int64_t gbr_star_num_blocks(const gbr_star *s);
int gbr_star_block_info(const gbr_star *s, int64_t block, char *name, size_t len, int64_t *ncols,
                        int64_t *nrows, int *is_loop);
int gbr_star_column_name(const gbr_star *s, int64_t block, int64_t col, char *name, size_t len);
/* Column `label` ("rlnDefocusU" or "_rlnDefocusU") of a block as doubles [nrows]. */
int gbr_star_column_double(const gbr_star *s, int64_t block, const char *label, double *out);
int gbr_star_value_string(const gbr_star *s, int64_t block, const char *label, int64_t row, char *buf,
                          size_t len);
void gbr_star_free(gbr_star *s);

/* Number of coarse directions / psi angles / translations of the sampling,
 * and the fine oversampling factors (HealpixSampling::NrDirections etc.). */
int gbr_sampling_sizes(const gbr_bundle *b, int64_t *ndir, int64_t *npsi, int64_t *ntrans,
                       int64_t *nover_rot, int64_t *nover_trans);

/* Debug read-back of the last batch, for parity tests: `what` selects
 *   0: coarse diff2 of particle i (absolute, double [R*T]; +inf = skipped)
 *   1: coarse weights of particle i (double [R*T])
 *   2: fine entries of particle i: int64 hidden indices [m] (what=2) and
 *   3: fine diff2 [m] (double), 4: fine weights [m] (double).
 * Returns the number of elements written, or a negative status. */
int64_t gbr_worker_debug_fetch(gbr_worker *w, int what, int64_t i, void *host, int64_t capacity);

/* AccBackprojector::getMdlData (src/acc/acc_backprojector_impl.h:109-138):
 * download the accumulated data (complex, interleaved) and weight volumes of
 * one class in double precision; dims via gbr_backprojector_dims. */
int gbr_backprojector_dims(const gbr_bundle *b, int64_t *xdim, int64_t *ydim, int64_t *zdim,
                           int64_t *yinit, int64_t *zinit, int64_t *r_max);
int gbr_backprojector_download(gbr_bundle *b, int64_t iclass, double *data, double *weight);

/* Replace one class's volumes (layout of gbr_backprojector_download), e.g.
 * with the sums over all ranks after MlOptimiserMpi::combineAllWeightedSums
 * (src/ml_optimiser_mpi.cpp:2028), before the reconstruction below. */
int gbr_backprojector_upload(gbr_bundle *b, int64_t iclass, const double *data, const double *weight);

/* --- reconstruction side of an iteration (FP64 on the device) ------------ */

/* BackProjector::enforceHermitianSymmetry (src/backprojector.cpp:2148-2165)
 * on one class's volumes: BackProjector::symmetrise for C1, as called by
 * MlOptimiser::symmetriseReconstructions (src/ml_optimiser.cpp:4729). */
int gbr_backprojector_symmetrise(gbr_bundle *b, int64_t iclass);

/* BackProjector::updateSSNRarrays (src/backprojector.cpp:1041-1204) of one
 * class: tau2_io [ori/2+1] is read and written; sigma2, data_vs_prior and
 * fourier_coverage [ori/2+1] are written (any may be NULL); fsc [ori/2+1] is
 * read when update_tau2_with_fsc.  CTF-premultiplied correction not
 * supported. */
int gbr_update_ssnr(gbr_bundle *b, int64_t iclass, double tau2_fudge, double *tau2_io, double *sigma2_out,
                    double *data_vs_prior_out, double *fourier_coverage_out, const double *fsc,
                    int update_tau2_with_fsc, int is_whole_instead_of_half);

typedef struct {
    int max_iter_preweight; /* gridding_nr_iter (--gridding_iter, 10)                    */
    int do_map;             /* add 1 / tau2 to the weights (MAP)                         */
    int skip_gridding;      /* 1 unless --dont_skip_gridding (relion_refine default 1)   */
    int minres_map;         /* --minres_map (5)                                          */
    double tau2_fudge;
    double normalise;       /* wsum_model.pdf_class[iclass] (used with gridding)         */
} gbr_recon_params;

/* Precision of the reconstruction-side transforms (gbr_reconstruct,
 * gbr_projector_from_map, gbr_fsc): FP64 (the reference's precision, the
 * default) or FP32 cuFFT; the weights, shell sums and maps stay FP64. */
enum { GBR_RECON_FP64 = 0, GBR_RECON_FP32 = 1 };
int gbr_recon_set_precision(gbr_bundle *b, int precision);

/* BackProjector::reconstruct (src/backprojector.cpp:1379-1872) of one
 * class's device volumes into the real-space map vol_out [ori]^ref_dim
 * (z, y, x; mymodel.Iref[iclass]); tau2 [ori/2+1] is read when do_map.
 * vol_out may be NULL: the map then stays on the device only, for a
 * following gbr_projector_from_map with vol = NULL. */
int gbr_reconstruct(gbr_bundle *b, int64_t iclass, const gbr_recon_params *p, const double *tau2, double *vol_out);

/* Projector::computeFourierTransformMap (src/projector.cpp:116-593, called by
 * MlModel::setFourierTransformMaps, src/ml_model.cpp:1505-1555) of the map
 * vol [ori]^ref_dim straight into class iclass's device projector, in place
 * of gbr_projector_upload: gridding pre-correction, zero padding, forward
 * transform, r <= r_max(current_size) kept; power_spectrum [ori/2+1]
 * (tau2_class when updating it) or NULL; min_ires <= 0: no high-pass.
 * vol = NULL: the device-resident map of the bundle's last gbr_reconstruct
 * (no other reconstruction-side call in between). */
int gbr_projector_from_map(gbr_bundle *b, int64_t iclass, const double *vol, int64_t current_size,
                           int do_gridding, int64_t min_ires, double *power_spectrum);

/* Read back one class's device projector (complex FP32, interleaved) and
 * its geometry: dims[7] = xdim, ydim, zdim, yinit, zinit, r_max, padding
 * factor.  data may be NULL to query the geometry only. */
int gbr_projector_download(gbr_bundle *b, int64_t iclass, float *data, int64_t *dims);

/* getFSC (src/fftw.cpp:481-525) of two maps [ori]^ref_dim -> fsc [ori/2+1]. */
int gbr_fsc(gbr_bundle *b, const double *map1, const double *map2, double *fsc);

/* Weighted sums accumulated since the last reset (added into `out`). */
int gbr_wsum_download(gbr_bundle *b, gbr_wsum *out);
/* 2D classification: wsum_model.prior_offset_class [K][2] accumulated since
 * the last reset, sum of weight * pixel * (old offset + translation)
 * (src/ml_optimiser.cpp:8668-8672, 9122-9126); added into `out`. */
int gbr_wsum_download_class_offsets(gbr_bundle *b, double *out);
/* Zero the volumes and weighted sums (start of a new iteration). */
int gbr_bundle_reset_wsum(gbr_bundle *b);

/* Accumulated timing of the worker's batches (ms): the ten E-step stages
 * (CUDA events on the worker's stream: prep, norm, cross term, coarse
 * weights, significance + job list, fine diff2, fine weights, weighted sums,
 * backprojection, read-back), then the input copies of each batch (device
 * time before the first stage), the host finalisation of the results, for
 * gbr_expect_images the image upload and the image preparation, and for
 * batches staged by gbr_stage_images the staging copy (copy stream) and the
 * compute stream's wait for it at the start of the call. */
int gbr_worker_stage_times(const gbr_worker *w, double *ms, int64_t n, int64_t *n_written);

/* Number of CUDA kernels this worker has launched (all batches so far). */
int gbr_worker_launch_count(const gbr_worker *w, int64_t *count);

/* CUDA graphs of the worker's coarse segment (GBR_OPT_GRAPH): how many were
 * captured and how many passes replayed one.  No counterpart in the
 * reference. */
int gbr_worker_graph_stats(const gbr_worker *w, int64_t *captures, int64_t *replays);

/* Measured FP32 FMA throughput of the device (TFLOP/s, register-resident
 * FMA chains on every SM): the roofline peak of the FP32 SIMT kernels.
 * No counterpart in the reference (a measurement utility). */
int gbr_measure_fp32_peak(int device, double *tflops);

/* Significance threshold of n rows of non-negative weights ([n][len],
 * device memory), with no memory allocation of any kind.  No counterpart in
 * the reference: it serves callers that cannot allocate device memory where
 * they need this step (code inside a no-allocation region, a host
 * application that only hands over device pointers, or a fixed up-front
 * memory budget).  For each row it returns the weight at which the
 * descending cumulative sum first exceeds adaptive_fraction x the row's sum
 * and the number of weights taken until then (the significance rule of
 * src/ml_optimiser.cpp:8120-8200 without --maxsig), in device arrays
 * threshold[n] and nr_significant[n]; work is queued on `stream` (a
 * cudaStream_t, NULL for the default stream) and runs asynchronously.
 * Limit: n <= 64 rows per call (larger n: GBR_ERR_INVALID).  A row with no
 * positive weight gets nr_significant 0 and threshold +inf.  Its working
 * memory is one fixed array of about 4.3 MB per GPU, held until the process
 * exits and shared by all calls: calls that overlap on the GPU race and must
 * be ordered by the caller.  The first call on a device looks up that
 * array's address and, with lazy module loading (the CUDA default), loads
 * the library's device code, which may allocate: make the first call on
 * each device before any stream capture and outside any region that must
 * not allocate; every later call allocates nothing. */
int gbr_significance_threshold_noalloc(const float *weights, int64_t n, int64_t len,
                                       double adaptive_fraction, float *threshold,
                                       uint32_t *nr_significant, void *stream);

/* ---- learned pose proposal ---------------------------------------------
 * No counterpart in the reference (its coarse search is exhaustive): a small
 * convolutional network that proposes the top-M coarse viewing directions of
 * a particle, trained on the device by the library's own forward, backward
 * and Adam kernels on views it generates from the bundle's current
 * reference (coarse projection table, one row per coarse orientation, so the
 * direction label is exact) with CTFs drawn from a pool and the model's noise.
 * Features: whitened coarse power |X|^2 / sigma2 over the active coarse
 * pixels in polar bins (nring rings x nangle angle bins over [0, pi)),
 * log(1 + mean) - log 2.  Layers: conv 3x5 (1 -> c1, ReLU), conv 3x5
 * (c1 -> c2, ReLU), both zero-padded along rings and circular along angles;
 * mean over angles; linear to one logit per HEALPix direction; softmax.
 * Parameters (float): W1 [c1][1][3][5], b1 [c1], W2 [c2][c1][3][5], b2 [c2],
 * W3 [c2*nring][ndir], b3 [ndir]. */
typedef struct gbr_posenet gbr_posenet;
typedef struct {
    int32_t nring;      /* rings 1..nring of the coarse image (<= coarse size / 2) */
    int32_t nangle;     /* angle bins over [0, pi) */
    int32_t c1, c2;     /* channels of the two convolutions (1..32) */
    int32_t max_batch;  /* particles or training views per launch */
    int32_t reserved;
    uint64_t seed;      /* weight initialisation and training views */
} gbr_posenet_desc;

/* The bundle must have its model arrays and projectors (the pose tables are
 * built here if needed); the network keeps a pointer to it and reads the
 * bundle's current tables, so destroy the network before the bundle.  3D
 * bundles only (GBR_ERR_UNSUPPORTED for 2D classification). */
int gbr_posenet_create(gbr_bundle *b, const gbr_posenet_desc *d, gbr_posenet **out);
int gbr_posenet_destroy(gbr_posenet *n);
/* parameter count, features per particle (nring * nangle), directions, active coarse pixels */
int gbr_posenet_sizes(const gbr_posenet *n, int64_t *nparams, int64_t *nfeat, int64_t *ndir, int64_t *npix);
/* active coarse pixels: (x, y) pairs [npix][2] and noise weights 1 / (2 sigma2) [npix] */
int gbr_posenet_pixels(const gbr_posenet *n, int32_t *xy, float *minv);
int gbr_posenet_get_params(const gbr_posenet *n, float *out);
int gbr_posenet_set_params(gbr_posenet *n, const float *in);
/* features [count][nfeat] of prepared images fimg (complex float
 * [count][current_size][current_size/2+1], the layout of gbr_particle_batch;
 * host or device memory, here and in gbr_posenet_block_probs /
 * gbr_posenet_propose) */
int gbr_posenet_features(gbr_posenet *n, const float *fimg, int64_t count, float *feat_out);
/* mean loss and its gradient for given features [count][nfeat] and target
 * distributions [count][ndir] (host; each target row sums to 1) */
int gbr_posenet_loss_grad(gbr_posenet *n, const float *feat, const float *target, int64_t count, double *loss,
                          float *grad_out);
/* `steps` Adam steps (learning rate lr) on `batch` generated views each; CTFs
 * drawn from ctf_pool (host, [n_pool][current_size][current_size/2+1], the
 * fctf layout); *loss_out = mean loss over the last min(steps, 20) steps */
int gbr_posenet_train(gbr_posenet *n, const float *ctf_pool, int64_t n_pool, int64_t steps, int64_t batch,
                      double lr, double *loss_out);
/* `steps` Adam steps on particle images with given target distributions:
 * fimg prepared images [count] (host, gbr_particle_batch layout), target
 * [count][ndir] (host; each row sums to 1), e.g. the E-step's own
 * posteriors over directions; mini-batches of `batch` consecutive particles,
 * cycling through the set; *loss_out as gbr_posenet_train */
int gbr_posenet_train_targets(gbr_posenet *n, const float *fimg, const float *target, int64_t count, int64_t steps,
                              int64_t batch, double lr, double *loss_out);
/* probability of each block of dirs_per_block consecutive directions
 * [count][ndir / dirs_per_block] under softmax(logits / temperature), for
 * prepared images fimg [count] (host or device) */
int gbr_posenet_block_probs(gbr_posenet *n, const float *fimg, int64_t count, int64_t dirs_per_block,
                            double temperature, float *out);
/* the m most probable blocks of dirs_per_block consecutive directions under
 * softmax(logits / temperature) [count][m] (most probable first, lower
 * index first among equals) and their summed probability [count], for
 * prepared images fimg [count] (host or device) */
int gbr_posenet_propose_blocks(gbr_posenet *n, const float *fimg, int64_t count, int64_t dirs_per_block,
                               double temperature, int64_t m, int32_t *blocks_out, float *mass_out);
/* top-m directions [count][m] (most probable first) and their probabilities */
int gbr_posenet_propose(gbr_posenet *n, const float *fimg, int64_t count, int64_t m, int32_t *dir_out,
                        float *prob_out);

/* delete MlOptimiserCuda / MlDeviceBundle (src/ml_optimiser.cpp:3840-3868). */
int gbr_worker_destroy(gbr_worker *w);
int gbr_bundle_destroy(gbr_bundle *b);

#ifdef __cplusplus
}
#endif
#endif /* GBRELION_H */
