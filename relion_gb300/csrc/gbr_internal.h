// gbr_internal.h -- internal types and kernel launch declarations of
// libgbrelion.  Kernels live in k_*.cu; the host driver in estep.cu.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <string>

namespace gbr {

// Error channel: every launch wrapper returns cudaError_t; the driver turns
// it into a gbr_status plus text (gbr_last_error).
struct Error {
    int status;
    std::string text;
};

// Set the text returned by gbr_last_error() on this thread.
void set_error_text(const std::string &msg);

// One active Fourier pixel of a 2D image of size s (FFTW half layout):
// logical frequency (x, y), its index in the full [s][s/2+1] image, and its
// resolution shell (Mresol, src/ml_optimiser.cpp:5784-5795).
struct PixelRef {
    int x, y;
    int full;   // index into [s][s/2+1]
    int shell;  // ROUND(sqrt(x^2+y^2)); -1 if excluded
};

// Padded Fourier volume geometry (Projector::data, src/projector.cpp:59-90).
struct VolGeom {
    int xdim, ydim, zdim, yinit, zinit, r_max, pad;
    int dim = 3;  // 3: padded 3D volume; 2: one padded 2D plane (2D classification)
};

// Per-particle state on the device (one per particle of the batch).
struct ParticleState {
    double c_coarse;     // highres_Xi2/2 + sum_k minv_c |X|^2 (coarse pixels)
    double c_fine;       // same for the fine pixels
    double sum_coarse;   // sum of coarse weights
    double sum_fine;     // sum of fine weights
    double sel_above;    // threshold search: weight sum above the current bucket
    double target;       // adaptive_fraction * sum of the pass being searched
    unsigned long long argmax_key;  // (weight bits << 32) | ~loop-order index
    unsigned int min_coarse;        // ordered-int encoding of min relative diff2
    unsigned int min_fine;
    unsigned int sel_prefix;        // threshold search: selected bit prefix
    unsigned int sel_count_above;   // elements strictly above the bucket
    float thr_coarse;               // significant weight of the coarse pass
    float thr_fine;                 // significant weight of the fine pass
    unsigned int nr_sign;           // significant count (coarse pass)
    float eps;                      // weights below eps cannot reach the threshold
    float xs;                       // coarse diff2 - min beyond which the weights of all
                                    // poses together stay below 1e-10 of the weight sum
    float po_min;                   // smallest normalised offset prior of the particle
};

// Fine-pass job: one (particle, significant coarse orientation).
struct FineJob {
    int p;          // particle in batch
    int r;          // coarse orientation (iclass*ndir + idir)*npsi + ipsi
    int n_t;        // significant coarse translations of this orientation
    int pad_;
    long long off;  // first fine entry of this job
};

// Histogram bin used by the threshold search.
struct HistBin {
    double sum;
    unsigned int count;
    unsigned int pad_;
};

constexpr int kHistBins = 4096;

// ---- launch wrappers (all asynchronous on `st`) -------------------------
// k_project.cu
cudaError_t launch_phase_table(float2 *out, const double *tx, const double *ty, int ntrans,
                               const PixelRef *pix, int npix, int ld, double ori_size, cudaStream_t st);
// Project n orientations (matrices Ainv*pad, row-major float[9]) of class
// volumes; orientation o uses class cls[o].  Output either interleaved
// (re,im) rows of `ld` floats (+ |P|^2 rows of `ld2` floats) or float2 rows.
// circ / mask (optional): per pixel the bit index of pixels exactly on the
// r_max circle (-1 elsewhere) and per orientation the bits of those the
// reference projects (Projector::project decides them in double precision).
// rout2 >= 0: pixels with x^2 + y^2 > rout2 are zero (the output image's
// circle, radius size / 2, as the reference fills it).
// texs: per-class texture objects of 3D CUDA array copies of the volumes
// (vol_texture_update; null: the linear volumes are read directly).
cudaError_t launch_project_rows(const float2 *const *vols, const VolGeom &g, const float *eul,
                                const int *cls, const int *orient_ids, int n_orient,
                                const PixelRef *pix, int npix, float *out_ri, int ld, float *out_p2,
                                int ld2, float2 *out_c, cudaStream_t st, const int *circ = nullptr,
                                const unsigned long long *mask = nullptr, int rout2 = -1,
                                const unsigned long long *texs = nullptr);
// A 3D CUDA array copy of a padded volume with a point-sampling texture
// object on it (the projector's fetch path); updated in place when the
// dimensions are unchanged.
struct VolTexture {
    cudaArray_t arr = nullptr;
    cudaTextureObject_t tex = 0;
    int x = 0, y = 0, z = 0;
};
cudaError_t vol_texture_update(VolTexture &t, const float2 *vol, const VolGeom &g, cudaStream_t st);
void vol_texture_release(VolTexture &t);

// FP32 FMA throughput probe (ms of one timed launch and its flop count).
cudaError_t launch_fp32_probe(float *ms, double *flops);

// k_tc.cu: tcgen05 BF16 coarse cross term (precision form).  Operand tiles
// are packed into [tiles][ktiles][bytes] images (sizes from tc_*_bytes).
// Norm term of the precision form on the tensor cores (kind::tf32, three-term
// split: FP32-level accuracy): A = |P|^2 table packed once per iteration,
// w = per-particle noise-weighted CTF^2 [n][ldw]; out[p][M].
size_t tc_norm_a_bytes(int M, int K);
size_t tc_norm_b_bytes(int N, int K);
cudaError_t launch_tc_norm_pack_a(const float *src, int lds, int M, int K, void *dst, cudaStream_t st);
cudaError_t launch_tc_norm(const void *Ablk, const float *w, int ldw, int M, int K, int nparticles, void *Bblk,
                           float *out, cudaStream_t st);
size_t tc_a_bytes(int M, int K2);
size_t tc_y_bytes(int N, int K2);
cudaError_t launch_tc_pack_a(const float *src, int lds, int M, int K2, void *dst, cudaStream_t st);
// Coarse cross term on tcgen05 (BF16, FP32 accumulation) with the diff2
// epilogue; with T >= 32 and rowmin non-null it also records the ordered
// minimum of every (particle, orientation) row (rowmin set to ~0 by the
// caller); with segmask non-null too (and T <= 960) it stores only the row
// segments within ps[p].xs of the running minimum and marks them in segmask
// (zeroed by the caller); the rest of `out` is left unwritten.
// Tile order and cache use of the coarse tensor-core kernel: group_m
// orientation tiles of 128 rows per group (0 = 32), keep_a reads the
// projection tiles with an L2 keep policy, pair runs the SM-pair kernel
// (cta_group::2, tiles of 256 orientations).
struct TcTuning {
    int group_m = 0;
    int keep_a = 0;
    int pair = 0;
};
cudaError_t launch_tc_diff2(const void *Ablk, void *Yblk, int M, int K2, const float2 *b, int ldb, const float2 *E,
                            int lde, int nparticles, int T, float *out, const float *norm, const float *pdf_orient,
                            ParticleState *ps, unsigned int *rowmin, unsigned int *segmask, cudaStream_t st,
                            const TcTuning &tune = TcTuning());
// Coarse cross term restricted to orientation blocks (precision form):
// blocks of NB consecutive rows of the projection table (NB % 32 == 0,
// NB <= 256, M % NB == 0) packed once per iteration; one work item per
// (particle, block) pair of `items`; needs T <= 128.  Scored rows are stored
// whole with their row minimum (rowmin, set to ~0 by the caller) and all
// segments marked in segmask (zeroed by the caller); other rows stay
// unscored.
size_t tc_blocks_bytes(int M, int K2, int NB);
size_t tc_yp_bytes(int nparticles, int K2);
cudaError_t launch_tc_pack_blocks(const float *src, int lds, int M, int K2, int NB, void *dst, cudaStream_t st);
cudaError_t launch_tc_blocks(const void *Bblk, int NB, void *Yp, int M, int K2, const float2 *b, int ldb,
                             const float2 *E, int lde, int nparticles, int T, const int2 *items, int nitems,
                             float *out, const float *norm, const float *pdf_orient, ParticleState *ps,
                             unsigned int *rowmin, unsigned int *segmask, cudaStream_t st);
// Read (and optionally clear) the tensor-core pipeline error flag.
cudaError_t tc_error_flag(int *flag, int reset);
cudaError_t tc_error_flag_async(int *host_flag, cudaStream_t st);

// k_gemm.cu: C[m][n] = sum_k A[m][k] * Bop[n][k], FP32 SIMT.
// Cross term + diff2 epilogue; output [p][M][T] relative to c_p, +inf where
// skipped; fine pass: mask = coarse significance [p][M/mdiv][W].
cudaError_t launch_gemm_diff2(const float *A, int lda, int M, int K2, const float2 *bimg, int ldb,
                              const float2 *phase, int ldp, int nparticles, int T, float *out,
                              const float *norm, const float *pdf_orient, const unsigned int *mask,
                              int mdiv, int tdiv, int W, ParticleState *ps, int fine, cudaStream_t st);
// C = A B^T (both K-contiguous rows, K padded to 16); C[m][n] or C[n][m].
cudaError_t launch_gemm_rows(const float *A, long long lda, int M, const float *B, long long ldb, int N,
                             int K, float *C, long long ldc, int trans_out, cudaStream_t st);
cudaError_t launch_gemm_bpimg(const float *W, int RF, int TF, int nparticles, const float *Zt, long long ldz,
                              int N2, float *img, long long ldi, cudaStream_t st);
cudaError_t launch_gemm_sigma_cross(const float *W, int RF, int TF, int nparticles, const float *P,
                                    long long ldp, int nf, const float2 *E, float2 *G, cudaStream_t st);
cudaError_t launch_gemm_sigma_norm(const float *Wrow, long long ldw, int nparticles, int RF, const float *P2,
                                   long long ldp2, int nf, float *S, cudaStream_t st);
cudaError_t launch_fine_normalize(float *w, int n, int R, int nOR, int nOT, int T, const ParticleState *ps,
                                  const double *pdat, const double *otx, const double *oty, double pixel,
                                  int ndir, int npsi, float *Wt, int ldwt, float *Wp, int ldwp, unsigned char *active,
                                  double *pacc, double *pdf_dir, double *pdf_cls, const double *class_prior,
                                  double *w_prior_off, cudaStream_t st);
cudaError_t launch_make_zt(const float *Cf, const float2 *Xnf, const float *minv_s, const float2 *E,
                           const double *pdat, int do_scale, int n, int TF, int nf, float *Zt, long long ldz,
                           float *CM, int ldcm, cudaStream_t st);
cudaError_t launch_shell_dense(int n, const float *S2P, const float2 *G, const float2 *Xf, const float *Cf,
                               const PixelRef *pf, int nf, int nshell, const double *pdat, int do_scale,
                               const unsigned char *dvp_mask, int K, double *pacc, double *shell,
                               cudaStream_t st);

// k_estep.cu
cudaError_t launch_prep(const float2 *X, const float *C, const double *pdat, int n, int full_npix,
                        const PixelRef *pc, int nc, const float *minv_c, int ldk_c,
                        const PixelRef *pf, int nf, int ldk_f, const float *minv_f, float *a_c, float2 *b_c,
                        float *a_f, float2 *b_f, float2 *Xf, float2 *Xnf, float *Cf,
                        const float2 *Xn, int do_scale, ParticleState *ps, cudaStream_t st);
cudaError_t launch_pdf_offset(const double *pdat, int n, const double *tx, const double *ty, int T,
                              double sigma2_offset, double pixel, float *pdf_off, double log_rt_orient,
                              ParticleState *ps, int KP, const double *class_prior, cudaStream_t st);
// Weights of per-particle segments [seg[p], seg[p+1]) of `vals` (in place).
// Coarse: element e of particle p has r = e / T, t = e % T.
// Fine: element e has job = ejob[e] and code = ecode[e].
cudaError_t launch_weights(float *vals, const long long *seg, int n, long long max_len, int coarse,
                           int T, const int *ejob, const unsigned int *ecode, const FineJob *jobs,
                           int nOR, int nOT, const float *pdf_orient, const float *pdf_off,
                           ParticleState *ps, HistBin *hist, cudaStream_t st, int add_sum = 1, int KP = 1, int rpc = 1,
                           const unsigned int *segmask = nullptr);
// Threshold search levels 0..2 (12, 12, 7 bits).  pass: 1 coarse, 2 fine
// (weights below (1 - fraction) * sum / segment length are skipped: they
// cannot reach the threshold), 0: no skipping.
cudaError_t launch_hist_refine(const float *vals, const long long *seg, int n, long long max_len,
                               int level, ParticleState *ps, HistBin *hist, cudaStream_t st,
                               int pass = 0, double fraction = 1.0, const long long *seg_end = nullptr,
                               long long n_total = 0);
// Coarse weights + FP64 sums + candidate lists (see k_weights_cand).
// Coarse weights, FP64 sums and candidate lists in one read of the diff2
// array; rows whose minimum (rowmin, may be null) lies more than ps[p].xs
// above the particle minimum are skipped without reading them.
cudaError_t launch_weights_cand(const float *vals, int n, int R, int T, const float *pdf_orient, float pdf_orient_min,
                                const float *pdf_off, double fraction, ParticleState *ps, unsigned int *cand_idx,
                                float *cand_w, unsigned int *cand_cnt, int cap, float *dense_out,
                                const unsigned int *rowmin, int KP, int rpc, const unsigned int *segmask,
                                int cand_buf, cudaStream_t st);
cudaError_t launch_cand_masks(const unsigned int *cand_idx, const float *cand_w, const unsigned int *cand_cnt,
                              int cap, int n, int R, int T, int W, const ParticleState *ps, unsigned int *mask,
                              int *cnt, cudaStream_t st);
// The three levels of the threshold search in one launch, one block per
// particle (segments up to kSelectFusedMax elements).
constexpr long long kSelectFusedMax = 1LL << 17;
cudaError_t launch_select_fused(const float *vals, const long long *seg, const long long *seg_end, int n,
                                long long n_total, int pass, double fraction, int coarse, ParticleState *ps,
                                cudaStream_t st);
cudaError_t launch_select(int n, int level, double adaptive_fraction, int coarse, ParticleState *ps,
                          HistBin *hist, cudaStream_t st);
cudaError_t launch_sig_masks(const float *w, int n, int R, int T, int W, const ParticleState *ps,
                             unsigned int *mask, int *cnt, cudaStream_t st);
// Fine-pass job list: jobs[] in (p, r) order for cnt > 0, seg[p] = first fine
// entry of particle p, seg[n] = total; sums holds 2 * ceil(n R / 1024) + 2
// values and ends with (number of jobs, number of fine entries).
// blocks of the job-list scan for tot (particle, orientation) counts; the
// totals (jobs, entries) land at sums[2 nblocks], sums[2 nblocks + 1]
long long fine_jobs_nblocks(long long tot);
// zero the mask words and counts of the job rows (job count read on the device)
cudaError_t launch_clear_job_rows(const FineJob *jobs, const long long *njobs_dev, long long njobs_max, int R, int W,
                                  unsigned int *mask, int *cnt, cudaStream_t st);
cudaError_t launch_fine_jobs(const int *cnt, int n, int R, int per, long long *sums, FineJob *jobs, long long *seg,
                             unsigned char *need_r, cudaStream_t st);
// Fine diff2 over a device work queue of (job, pixel range) items: the job
// count is read on the device (njobs_dev; njobs_max sizes the arrival
// counters), nsplit = fine_diff2_nsplit(nf) ranges per job, head / arrive
// are zeroed by the launcher, part holds [nfine][nsplit] and npart
// [njobs][8][nsplit] floats.
int fine_diff2_nsplit(int nf);
cudaError_t launch_fine_diff2(const FineJob *jobs, const long long *njobs_dev, long long njobs_max, int nsplit,
                              unsigned long long *head, int *arrive, float *part, float *npart,
                              const unsigned int *mask, int R, int T, int W, int nOR, int nOT, const float2 *projf,
                              int ldpf, const float2 *b_f, const float *a_f, int nf, const float2 *phase_f, float *d,
                              int *ejob, unsigned int *ecode, ParticleState *ps, cudaStream_t st);
struct WsumArgs {
    const FineJob *jobs;
    long long njobs;
    const unsigned int *mask;
    int R, T, W, nOR, nOT, nf, ldpf, nshell, ndir, npsi, K;
    const float *w;            // fine weights
    const ParticleState *ps;
    const float2 *projf;       // [R*nOR][nf]
    const float2 *Xf, *Xnf;    // [p][nf]
    const float *Cf;           // [p][nf] (scaled CTF)
    const float *minv_store;   // [nf]
    const PixelRef *pf;
    const float2 *phase_f;     // [T*nOT][nf]
    const double *otx, *oty;   // [T*nOT] fine translations in pixels
    const double *pdat;        // [p][8]
    double pixel;
    int do_scale;
    const unsigned char *dvp_mask;  // [K][nshell] data_vs_prior > 3 (scale corr.)
    float2 *bpimg;             // [R*nOR][nf]
    float *bpw;                // [R*nOR][nf]
    unsigned char *active;     // [R*nOR]
    double *shell;             // [p][nshell]
    double *pacc;              // [p][8]: sumw, sigma2_offset, XA, AA
    double *pdf_dir;           // [K*ndir]
    double *pdf_cls;           // [K]
    const double *class_prior; // [K][2] 2D classification: per-class offset prior, else null
    double *w_prior_off;       // [K][2] 2D: sum w pixel (old offset + shift), else null
    // direct insertion (bp_direct): each job's weighted slices go straight
    // into the staging volumes (no slice accumulators, no backprojection pass)
    int bp_direct;
    const float *eul_f;        // [R*nOR][9]
    float4 *const *stage;      // [K] staging volumes
    VolGeom bg;
    const int *circ;           // [nf] r_max-circle pixel bit, -1 off the circle (or null)
    const unsigned long long *cmask;  // [R*nOR] circle pixels inserted per slice (or null)
};
cudaError_t launch_wsum(const WsumArgs &a, cudaStream_t st);
// Image preparation (getFourierTransformsAndCtfs) of n real-space images of
// N x N pixels into the E-step inputs of the current size `cur`.
struct PrepImagesArgs {
    int n, N, cur;
    const float *images;   // [n][N][N] row y, column x (device)
    const int *shift;      // [n][2] rounded old offset (dx, dy)
    const float *factor;   // [n] norm-correction factor (1 without --norm)
    const double *ctf;     // [n][6] defU, defV, defAngle, Bfac, scale, phase shift
    double pixel, kV, Cs, Q0, mask_radius, mask_width;
    float *A, *B;          // [n][N][N] scratch: shifted, masked
    float2 *FA, *FB;       // [n][N][N/2+1] scratch: their transforms
    double *bg;            // [n][2] scratch: mask background sums (sum w v, sum w)
    float *W;              // [N][N] background weights of the soft mask
    int mask_fresh;        // 1: (re)compute W for this geometry
    long long fft_plan;    // batched N x N R2C plan (make_fft_plan)
    float2 *fimg, *fimg_nomask;  // [n][cur][cur/2+1]
    float *fctf;                 // [n][cur][cur/2+1]
    double *power, *xi2;         // [n][N/2+1], [n]
};
cudaError_t launch_prepare_images(const PrepImagesArgs &a, cudaStream_t st);
int make_fft_plan(int N, int batch, long long *plan_out);
void destroy_fft_plan(long long plan);

cudaError_t launch_compact_flags(const unsigned char *flags, int n, int *list, int *count,
                                 cudaStream_t st);
// circ / mask: as launch_project_rows, for the backprojection's own test
// (BackProjector::backproject2Dto3D decides the r_max-circle pixels in double
// precision by its per-row ellipse bounds and its 3D radius check).
// Trilinear insertion of the active slices into the FP32 staging volumes
// (float4 re, im, weight, 0 per voxel, one per class); launch_bp_flush adds
// a staging volume into the FP64 data / weight volumes and clears it.
cudaError_t launch_backproject(const int *list, const int *count, int max_list, const float *eul_f, int nOR,
                               const int *cls_of_r, float2 *bpimg, float *bpw, const PixelRef *pf, int nf,
                               const VolGeom &g, float4 *const *stage, unsigned char *active, cudaStream_t st,
                               const int *circ = nullptr, const unsigned long long *mask = nullptr);
cudaError_t launch_bp_flush(float4 *stage, double2 *data, double *weight, const VolGeom &g, cudaStream_t st);
cudaError_t launch_gather_pdat(const double *old_offset, const double *prior, const double *xi2,
                               const double *norm, const double *scale, int n, double *pdat, cudaStream_t st);
cudaError_t launch_cand_seg(const unsigned int *cnt, int n, int cap, long long *seg, cudaStream_t st);

}  // namespace gbr

// Reconstruction side of an iteration (k_recon.cu).  Host entry points run
// on the legacy default stream and synchronise; they return 0 or a
// gbr_status with the text set through set_error_text.
namespace gbr {
struct ReconWork;  // device scratch and cached double-precision FFT plans
ReconWork *recon_work_create();
void recon_work_destroy(ReconWork *w);
// transforms in FP32 (1) or FP64 (0, default)
void recon_set_fp32(ReconWork *w, int fp32);
struct ReconParams {
    int max_iter_preweight, do_map, skip_gridding, minres_map;
    double tau2_fudge, normalise;
};
// Projector::initialiseData(current_size) geometry for a padded reference
VolGeom projector_geometry(int ori, int dim, int pad, int current_size);
int recon_symmetrise(double2 *data, double *weight, const VolGeom &g);
int recon_update_ssnr(ReconWork *w, const double *weight, const VolGeom &g, int ori, double tau2_fudge,
                      double *tau2_io, double *sigma2_out, double *dvp_out, double *cov_out, const double *fsc,
                      int upd, int whole);
int recon_reconstruct(ReconWork *w, const double2 *data, const double *weight, const VolGeom &g, int ori,
                      const ReconParams &p, const double *tau2_host, double *vol_host);
int recon_projector_from_map(ReconWork *w, const double *vol_host, int ori, int dim, int pad, const VolGeom &pg,
                             int do_gridding, int min_ires, float2 *proj, double *power_host);
int recon_fsc(ReconWork *w, const double *m1, const double *m2, int ori, int dim, double *fsc_host);
}  // namespace gbr

// Pose-proposal network (k_posenet.cu).  Parameter offsets into one float
// array; activations [B][C][H][W] with H rings and W angle bins.
namespace gbr {
struct PnDims {
    int B = 0, H = 0, W = 0, C1 = 0, C2 = 0, ND = 0;
    long long o_w1 = 0, o_b1 = 0, o_w2 = 0, o_b2 = 0, o_w3 = 0, o_b3 = 0, nparams = 0;
};
cudaError_t pn_gen(const float *proj, int lda, const PixelRef *pix, int npix, const float *minv,
                   const float *ctf_pool, int full_npix, int n_pool, long long R, int NP, int ND, uint64_t seed,
                   int B, float *v, int *label, cudaStream_t st);
cudaError_t pn_power(const float2 *fimg, int full_npix, const PixelRef *pix, int npix, const float *minv, int B,
                     float *v, cudaStream_t st);
cudaError_t pn_bin(const float *v, int npix, const int *bin, const float *inv_cnt, int nbins, int B, float *feat,
                   cudaStream_t st);
cudaError_t pn_forward(const PnDims &d, const float *params, const float *feat, float *a1, float *a2, float *h,
                       float *logits, cudaStream_t st);
// scratch of pn_loss_backward: pn_backward_scratch(d) floats
size_t pn_backward_scratch(const PnDims &d);
cudaError_t pn_loss_backward(const PnDims &d, const float *params, const float *feat, const float *a1,
                             const float *a2, const float *h, const float *logits, const int *label,
                             const float *target, float *dl, float *loss, float *d2, float *d1, float *grad,
                             float *scratch, cudaStream_t st);
cudaError_t pn_adam(float *p, const float *g, float *m, float *v, long long n, float lr, int t, cudaStream_t st);
cudaError_t pn_topm(const float *logits, int N, int M, int B, int *idx, float *prob, cudaStream_t st);
// the m most probable of nb block probabilities per particle and their sum
cudaError_t pn_top_blocks(const float *probs, int nb, int m, int B, int *idx, float *mass, cudaStream_t st);
cudaError_t pn_block_probs(const float *logits, int N, int dpb, float temperature, int B, float *out,
                           cudaStream_t st);
}  // namespace gbr
