// estep.cu -- host side of libgbrelion: the C ABI of include/gbrelion.h,
// the per-iteration device tables (MlDeviceBundle) and the batched E-step
// driver (MlOptimiserCuda::doThreadExpectationSomeParticles).
//
// One batch runs as: particle preparation -> coarse norm GEMM -> coarse
// cross GEMM (diff2) -> weights + threshold search -> significance masks and
// fine jobs -> fine projections (cached per iteration) -> fine diff2 ->
// weights + threshold search -> weighted sums -> backprojection.  The host
// synchronises once per batch, after the coarse significance, to size the
// fine pass, and once at the end to read the per-particle results.
#include "../../include/gbrelion.h"
#include "gbr_internal.h"
#include "sampling.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <atomic>
#include <string>
#include <vector>

using namespace gbr;

namespace {

thread_local std::string g_last_error;

// Particles whose backprojected insertions the FP32 staging volumes collect
// before they are added into the FP64 volumes (GBR_OPT_BP_FLUSH).  Each voxel
// inside the insertion sphere takes ~70 insertions per 512 particles at
// current size 256, so an FP32 sum of 2048 particles carries ~1e-6 relative
// rounding; the FP64 volumes accumulate the flushes.
constexpr int kBpFlushDefault = 2048;

int fail(int status, const std::string &msg) {
    g_last_error = msg;
    return status;
}

#define GBR_CUDA(expr)                                                                     \
    do {                                                                                   \
        cudaError_t e_ = (expr);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            int st_ = (e_ == cudaErrorMemoryAllocation) ? GBR_ERR_OOM : GBR_ERR_CUDA;      \
            return fail(st_, std::string(#expr) + ": " + cudaGetErrorString(e_));          \
        }                                                                                  \
    } while (0)

#define GBR_LOCK(bundle) std::lock_guard<std::recursive_mutex> lock_((bundle)->mu)

// Keys of the CUDA graph of a worker's coarse segment (run_coarse): a graph
// replays only while the kernels' pointers and by-value arguments are the
// captured ones.  g_api_gen is bumped by every call that changes model,
// tables, optics or worker settings; g_alloc_count by every (re)allocation
// or release of a device or pinned buffer (a segment run that allocated is
// not captured on its next call).
std::atomic<unsigned long long> g_api_gen{0};
std::atomic<unsigned long long> g_alloc_count{0};

template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n) {
        o.p = nullptr;
        o.n = 0;
    }
    ~DevBuf() { release(); }
    void release() {
        if (p) {
            cudaFree(p);
            ++g_alloc_count;
        }
        p = nullptr;
        n = 0;
    }
    // grow to at least m elements (contents discarded)
    cudaError_t reserve(size_t m) {
        if (m <= n && p) return cudaSuccess;
        release();
        size_t bytes = std::max<size_t>(m, 1) * sizeof(T);
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e == cudaSuccess) n = std::max<size_t>(m, 1);
        ++g_alloc_count;
        return e;
    }
    cudaError_t upload(const T *h, size_t m) {
        cudaError_t e = reserve(m);
        if (e != cudaSuccess) return e;
        return cudaMemcpy(p, h, m * sizeof(T), cudaMemcpyHostToDevice);
    }
    cudaError_t zero(cudaStream_t st = 0) { return cudaMemsetAsync(p, 0, n * sizeof(T), st); }
};

// Page-locked host buffer: device-to-host copies into it stay asynchronous.
template <class T>
struct PinnedBuf {
    T *p = nullptr;
    size_t n = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf &) = delete;
    PinnedBuf &operator=(const PinnedBuf &) = delete;
    ~PinnedBuf() { release(); }
    void release() {
        if (p) {
            cudaFreeHost(p);
            ++g_alloc_count;
        }
        p = nullptr;
        n = 0;
    }
    cudaError_t reserve(size_t m) {
        if (m <= n && p) return cudaSuccess;
        release();
        void *q = nullptr;
        ++g_alloc_count;
        cudaError_t e = cudaMallocHost(&q, std::max<size_t>(m, 1) * sizeof(T));
        if (e == cudaSuccess) {
            p = static_cast<T *>(q);
            n = std::max<size_t>(m, 1);
        }
        return e;
    }
};

inline int pad16(int v) { return (v + 15) / 16 * 16; }

// Resolution-shell index (Mresol) of pixel (x, y) of an image of size s.
inline int shell_of(int x, int y, int s) {
    const int ires = iround(std::sqrt((double)(x * x + y * y)));
    if (ires < s / 2 + 1 && !(x == 0 && y < 0)) return ires;
    return -1;
}

inline float ord2f_host(unsigned int u) {
    unsigned int b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    float f;
    std::memcpy(&f, &b, 4);
    return f;
}

enum Stage { ST_PREP = 0, ST_NORM, ST_CROSS, ST_WCOARSE, ST_SIG, ST_PROJF, ST_FINE, ST_WFINE,
             ST_WSUM, ST_BP, ST_N };

}  // namespace

void gbr::set_error_text(const std::string &msg) { g_last_error = msg; }

struct gbr_bundle {
    // every call that runs work on the bundle's shared state (E-step,
    // image preparation, volumes, model arrays) holds this lock, so workers
    // of one bundle may be driven from several threads (as the reference's
    // threads drive their MlOptimiserCuda on one MlDeviceBundle): their
    // calls are serialised
    std::recursive_mutex mu;
    gbr_model_desc d{};
    int device = 0;
    PoseGrid grid;
    long K = 0, ND = 0, NP = 0, T = 0, R = 0, nOR = 0, nOT = 0, RF = 0, TF = 0;
    int nshell = 0;  // ori/2+1
    int cur = 0, crs = 0, full_npix = 0;
    // pixel lists
    std::vector<PixelRef> pc_h, pf_h;
    int nc = 0, nf = 0, ldk_c = 0, lda_c = 0;
    double logsigma2 = 0.;
    size_t budget = 0;
    // model arrays (host copies)
    std::vector<double> sigma2, pdf_class, pdf_dir, dvp;
    bool have_arrays = false;
    // image preparation (gbr_bundle_set_optics)
    gbr_optics_desc optics{};
    bool have_optics = false;
    // 2D classification (ref_dim 2): per-class offset priors and their sums
    bool is2d = false;
    int KP = 1;  // offset-prior rows per particle: K in 2D, 1 in 3D
    std::vector<double> class_prior_h;
    DevBuf<double> class_prior, w_prior_off;
    // projector
    VolGeom pg{}, bg{};
    std::vector<DevBuf<float2>> vol;
    std::vector<char> have_vol;
    DevBuf<const float2 *> vols_d;
    std::vector<gbr::VolTexture> vtex;   // 3D: array copies of the volumes for the projector's texture fetches
    DevBuf<unsigned long long> texs_d;
    // backprojector (FP64)
    std::vector<DevBuf<double2>> bp_data;
    std::vector<DevBuf<double>> bp_weight;
    std::vector<DevBuf<float4>> bp_stage;  // insertions since the last flush (FP32), flushed into bp_data / bp_weight
    DevBuf<float4 *> bps_ptrs;
    long long staged = 0;                  // particles inserted into bp_stage since the last flush
    size_t bp_vox = 0;
    // iteration tables
    bool tables_ready = false;
    DevBuf<PixelRef> pc, pf;
    DevBuf<float> minv_c, minv_f, minv_store;
    DevBuf<float> eul_c, eul_f;
    // pixels exactly on the r_max circle: bit index per pixel (-1 elsewhere)
    // and per orientation the bits of those the reference projects /
    // backprojects (3D; decided on the host as the reference decides them)
    DevBuf<int> pcirc_c, pcirc_f, bcirc_f;
    DevBuf<unsigned long long> pmask_c, pmask_f, bmask_f;
    bool use_circ = false;
    DevBuf<int> cls_c, cls_f, cls_of_r;
    DevBuf<float> pdf_orient;
    float pdf_orient_min = 0.f;  // smallest non-zero normalised pdf_orient
    float pdf_orient_max = 0.f;
    DevBuf<double> tx, ty, otx, oty;
    std::vector<double> otx_h, oty_h;
    DevBuf<float2> phase_c, phase_f;
    DevBuf<float> proj_c, proj2_c;
    DevBuf<unsigned char> proj_c_tc;  // precision form: BF16 A tiles (tcgen05 smem image)
    DevBuf<unsigned char> proj2_c_tf; // precision form: TF32 split tiles of |P|^2 (norm term)
    DevBuf<unsigned char> proj_c_blk; // orientation-block tiles of the BF16 table (restricted coarse pass)
    bool blk_ready = false;
    DevBuf<float> proj_f, proj2_f;  // all oversampled orientations: [RF][lda_f], [RF][ldk_f]
    int ldk_f = 0, lda_f = 0;
    DevBuf<float2> bpimg;
    DevBuf<float> bpw;
    DevBuf<unsigned char> active;
    DevBuf<unsigned char> dvp_mask;
    // weighted sums
    DevBuf<double> w_pdf_cls, w_pdf_dir;
    std::vector<double> w_sigma2;
    double w_sigma2_offset = 0, w_sumw_group = 0, w_LL = 0, w_ave_Pmax = 0, w_avg_norm = 0, w_XA = 0,
           w_AA = 0;
    // reconstruction side: scratch and FFT plans, created on first use
    gbr::ReconWork *recon = nullptr;
    ~gbr_bundle() { gbr::recon_work_destroy(recon); }
};

struct gbr_worker {
    gbr_bundle *b = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[ST_N + 1] = {};
    double stage_ms[ST_N + 6] = {};  // device stages, input copies, host finalisation,
                                     // image upload and image preparation
    cudaEvent_t ev_in = nullptr;     // start of the batch's input copies
    cudaEvent_t ev_img[3] = {};      // image upload start, preparation start, end
    // image batches staged ahead (gbr_stage_images): two device slots filled on
    // a copy stream while the compute stream works on the previous batch
    struct StageSlot {
        DevBuf<float> img;
        cudaEvent_t start = nullptr, ready = nullptr, consumed = nullptr;
        const float *host = nullptr;
        int64_t n = 0;
        size_t npx = 0;
        long long seq = 0;  // staging order: matching slots are used oldest first
        bool valid = false;    // holds (or will hold) the images of (host, n)
        bool pending = false;  // requested, copy not yet issued
        bool used = false;     // consumed has been recorded at least once
    } stage[2];
    int stage_next = 0;
    long long stage_seq = 0;
    cudaEvent_t ev_call = nullptr;  // start of a gbr_expect_images call using a staged slot
    cudaEvent_t ev_inputs = nullptr;  // the call's host-to-device input copies are done
    cudaStream_t st_copy = nullptr;
    int debug = 0;
    int cap = 0;  // particles the batch buffers hold
    long long launches = 0;  // kernels launched by this worker
    // inputs
    DevBuf<float2> X, Xn;
    DevBuf<float> C;
    DevBuf<double> pdat, power;
    // prepared
    DevBuf<float> a_c, a_f, Cf;
    DevBuf<float2> b_c, b_f, Xf, Xnf;
    DevBuf<ParticleState> ps;
    DevBuf<float> pdf_off, nrm, vals;
    DevBuf<long long> seg_c, seg_f;
    DevBuf<HistBin> hist;
    DevBuf<unsigned int> mask;
    DevBuf<int> cnt;
    DevBuf<long long> scan_tmp;
    // fine-pass work queue: head counter, per-job arrivals, partial sums
    DevBuf<unsigned long long> fq_head;
    DevBuf<int> fq_arrive;
    DevBuf<float> fq_part, fq_npart;
    DevBuf<FineJob> jobs;
    DevBuf<unsigned char> need_r;
    DevBuf<int> proj_ids, act_list, act_count;
    DevBuf<float> fd;
    DevBuf<int> ejob;
    DevBuf<unsigned int> ecode;
    DevBuf<double> shell, pacc;
    DevBuf<unsigned char> ytc;  // precision form: BF16 B tiles of the batch
    DevBuf<unsigned char> wtf;  // precision form: TF32 split tiles of the norm weights
    // coarse significance candidates
    int cand_cap = 0;
    DevBuf<unsigned int> cand_idx, cand_cnt;
    DevBuf<float> cand_w, dense_dbg;
    DevBuf<unsigned int> rowmin;           // [p][R] row minima of the tensor-core coarse pass
    DevBuf<unsigned int> segmask;          // [p][R] row segments it stored (sparse writes)
    DevBuf<long long> cand_seg;  // [2n]: begins, ends
    // page-locked read-back of the batch (counts, job totals, results) and
    // the host copies of device-resident metadata
    PinnedBuf<unsigned int> h_ccnt;
    PinnedBuf<long long> h_totals, h_segf;
    PinnedBuf<int> h_tcflag;  // tensor-core pipeline error flag of the call
    PinnedBuf<ParticleState> h_ps;
    PinnedBuf<double> h_shell, h_pacc, h_pdat, h_power;
    // image preparation: inputs, scratch, FFT plan and the prepared batch
    DevBuf<float> pi_images, pi_A, pi_B, pi_factor, pi_fctf, pi_W;
    double pi_W_key[3] = {0., 0., 0.};  // N, radius, width of the cached mask weights
    DevBuf<float2> pi_FA, pi_FB, pi_fimg, pi_fnm;
    DevBuf<double> pi_bg, pi_ctf, pi_power, pi_xi2, pi_off, pi_prior, pi_norm, pi_scale;
    DevBuf<int> pi_shift;
    long long fft_plan = -1;
    int fft_N = 0, fft_batch = 0;
    // dense fine pass
    int fine_mode = 0;  // 0: by significant density, 1: always dense, 2: always sparse
    int coarse_rows = 0;  // 0: skip far coarse rows by their minimum (tensor-core pass), 1: read all rows
    int cand_cap_max = 1 << 16;  // candidate-list entries per particle (GBR_OPT_CAND_CAP)
    int cand_buf = 0;            // block-local candidate buffer used (GBR_OPT_CAND_BUF; 0 = all of it)
    int last_dense = 0;
    DevBuf<float> Wt, Wp, Zt, CM, S2P, fnrm;
    DevBuf<float2> G;
    // coarse pass restricted to orientation blocks (gbr_expect_batch_blocks):
    // the caller's [n_all][restrict_m] block lists, the first particle of the
    // current pass and the pass's (particle, block) work items
    const int32_t *restrict_blocks = nullptr;
    int64_t restrict_m = 0;
    int pass_p0 = 0;
    long long last_items = 0;  // work items of the last restricted pass
    PinnedBuf<int2> items_h;
    DevBuf<int2> items_d;
    DevBuf<unsigned char> ytp;  // per-particle BF16 Y tiles of the restricted pass
    int batch_cap = 0;           // particles per pass (GBR_OPT_BATCH_CAP; 0 = from the budget)
    int bp_flush = kBpFlushDefault;  // flush the staging volumes at this many particles (GBR_OPT_BP_FLUSH)
    int bp_direct = 0;    // sparse fine pass: weighted slices inserted by the weighted sums (GBR_OPT_BP_DIRECT)
    int last_direct = 0;  // the last pass inserted its slices directly
    // CUDA graph of the coarse segment (run_coarse; GBR_OPT_GRAPH)
    int use_graph = 1;
    cudaGraphExec_t gexec = nullptr;
    unsigned long long buf_gen = 0;  // bumped when the worker's batch buffers are reallocated
    bool masks_clean = false;        // mask / cnt are all zero (cleared after each pass)
    struct GraphKey {
        int n = -1;
        unsigned long long api = 0, buf = 0;
        bool operator==(const GraphKey &o) const { return n == o.n && api == o.api && buf == o.buf; }
    } g_key, warm_key;
    int g_launches = 0;
    long long g_captures = 0, g_replays = 0;
    TcTuning tc_tune;            // GBR_OPT_TILE_GROUP, GBR_OPT_KEEP_A, GBR_OPT_PAIR
    int pass_cap = 0;            // particles per pass of the current call
    // debug copies of the last call, one entry per pass (gbr_worker_debug_fetch)
    struct DbgPass {
        int n = 0;                        // particles of the pass
        int dense = 0;                    // fine pass ran as dense contractions
        int sparse = 0;                   // coarse diff2 stored only near the running minimum
        std::vector<float> coarse;        // relative coarse diff2 [n][R*T]
        std::vector<unsigned int> segmask;  // [n][R] stored 32-column segments (sparse)
        std::vector<float> wcoarse;       // coarse weights [n][R*T]
        std::vector<double> cc, cf;       // per-particle diff2 constants (coarse, fine)
        std::vector<float> fine, wfine;
        std::vector<int> ejob;
        std::vector<unsigned int> ecode;
        std::vector<FineJob> jobs;
        std::vector<long long> segf;
    };
    std::vector<DbgPass> dbg;
    int dbg_n = 0;                        // particles of the last call
};

namespace {

// ---- the reference's inside-r_max decisions, in double precision ---------
// Pixels strictly inside or outside the r_max circle are decided exactly by
// integers (|Ainv (x, y, 0)|^2 = pad^2 (x^2 + y^2) for a rotation); for the
// few pixels exactly on the circle the reference's double-precision tests
// decide, by the last bits of its inverted rotation matrix, and are restated
// here with the same operations (this file is compiled without contraction
// of multiply-adds).
inline int r_ceil(double x) { return (x == (int)x) ? (int)x : ((x > 0) ? (int)(x + 1) : (int)x); }
inline int r_floor(double x) { return (x == (int)x) ? (int)x : ((x > 0) ? (int)x : (int)(x - 1)); }

// Matrix2D<RFLOAT>::inv of a 3x3 matrix (src/matrix2d.h:1098-1125: adjugate
// over determinant) times the padding factor (src/projector.cpp:638).
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

// Projector::project keeps pixel (x, y) unless r_ref_2 > r_max_ref_2
// (src/projector.cpp:665-672).
bool ref_projects(const double Ai[9], int x, int y, int r_max_ref_2) {
    const double xp = Ai[0] * x + Ai[1] * y, yp = Ai[3] * x + Ai[4] * y, zp = Ai[6] * x + Ai[7] * y;
    return !(xp * xp + yp * yp + zp * zp > r_max_ref_2);
}

// BackProjector::backproject2Dto3D inserts pixel (x, y) when x lies within
// the row's ellipse bounds (src/backprojector.cpp:84-92, :150-160) and
// r2_3D <= max_r2 (:188); no Ewald sphere, identity magnification.
bool ref_inserts(const double Ai[9], int x, int y, int max_r2, int sh) {
    const double AtA_xx = Ai[0] * Ai[0] + Ai[3] * Ai[3] + Ai[6] * Ai[6];
    const double AtA_xy = Ai[0] * Ai[1] + Ai[3] * Ai[4] + Ai[6] * Ai[7];
    const double AtA_yy = Ai[1] * Ai[1] + Ai[4] * Ai[4] + Ai[7] * Ai[7];
    const double AtA_xy2 = AtA_xy * AtA_xy;
    const double discr = AtA_xy2 * y * y - AtA_xx * (AtA_yy * y * y - max_r2);
    if (discr < 0.) return false;
    const double dd = std::sqrt(discr) / AtA_xx;
    const double q = -AtA_xy * y / AtA_xx;
    const int first_allowed_x = y < 0 ? 1 : 0;
    const int first_x = std::max(r_ceil(q - dd), first_allowed_x), last_x = std::min(r_floor(q + dd), sh - 1);
    if (x < first_x || x > last_x) return false;
    const double xp = Ai[0] * x + Ai[1] * y, yp = Ai[3] * x + Ai[4] * y, zp = Ai[6] * x + Ai[7] * y;
    return !(xp * xp + yp * yp + zp * zp > max_r2);
}

// Bit index of each pixel of a list that lies exactly on the circle
// pad^2 (x^2 + y^2) == r2 (-1 elsewhere); the number of such pixels.
int circle_bits(const std::vector<PixelRef> &px, long pad, long r2, std::vector<int> &bit) {
    bit.assign(px.size(), -1);
    int nb = 0;
    for (size_t j = 0; j < px.size(); ++j)
        if (pad * pad * ((long)px[j].x * px[j].x + (long)px[j].y * px[j].y) == r2) bit[j] = nb++;
    return nb;
}

// The pixels of a list that lie on the circle (bit >= 0), in bit order.
std::vector<int> circle_pixels(const std::vector<int> &bit) {
    std::vector<int> idx;
    for (size_t j = 0; j < bit.size(); ++j)
        if (bit[j] >= 0) idx.push_back((int)j);
    return idx;
}

// Bit mask of the circle pixels (indices `on`) that the reference projects
// (or inserts) for the inverse rotation Ai.
unsigned long long circle_mask(const std::vector<PixelRef> &px, const std::vector<int> &on,
                               const std::vector<int> &bit, const double Ai[9], bool backproject, int r2, int sh) {
    unsigned long long m = 0ull;
    for (int j : on)
        if (backproject ? ref_inserts(Ai, px[j].x, px[j].y, r2, sh) : ref_projects(Ai, px[j].x, px[j].y, r2))
            m |= 1ull << bit[j];
    return m;
}

int build_tables(gbr_bundle *b) {
    if (b->tables_ready) return GBR_OK;
    ++g_api_gen;
    b->blk_ready = false;
    if (!b->have_arrays) return fail(GBR_ERR_STATE, "model arrays not set (gbr_model_set_arrays)");
    for (long k = 0; k < b->K; ++k)
        if (!b->have_vol[k]) return fail(GBR_ERR_STATE, "reference of class " + std::to_string(k) + " not uploaded");
    const gbr_model_desc &d = b->d;
    const double pix = d.pixel_size;
    // ---- pixel lists and noise weights (src/ml_optimiser.cpp:6880-6892) ----
    auto minv_of = [&](int shell) -> double {
        if (shell > 0 && shell < d.sigma2_len) return 1. / (d.sigma2_fudge * b->sigma2[shell]);
        return 0.;
    };
    b->pc_h.clear();
    std::vector<float> mc;
    for (int i = 0; i < b->crs; ++i) {
        const int X = b->crs / 2 + 1;
        const int y = (i < X) ? i : i - b->crs;
        for (int x = 0; x < X; ++x) {
            const int sh = shell_of(x, y, b->crs);
            const double m = minv_of(sh);
            if (m > 0.) {
                const int yi = y < 0 ? y + b->cur : y;  // row in the fine image
                b->pc_h.push_back(PixelRef{x, y, yi * (b->cur / 2 + 1) + x, sh});
                mc.push_back((float)(0.5 * m));
            }
        }
    }
    b->pf_h.clear();
    std::vector<float> mf, ms;
    for (int i = 0; i < b->cur; ++i) {
        const int X = b->cur / 2 + 1;
        const int y = (i < X) ? i : i - b->cur;
        for (int x = 0; x < X; ++x) {
            const int sh = shell_of(x, y, b->cur);
            if (sh < 0) continue;
            b->pf_h.push_back(PixelRef{x, y, i * X + x, sh});
            const double m = minv_of(sh);
            mf.push_back((float)(0.5 * m));
            double mst = m;
            if (x == 0 && y == 0) mst = 1. / (d.sigma2_fudge * b->sigma2[0]);  // :8301
            ms.push_back(d.do_map ? (float)mst : 1.f);
        }
    }
    b->nc = (int)b->pc_h.size();
    b->nf = (int)b->pf_h.size();
    b->ldk_c = pad16(std::max(b->nc, 1));
    b->lda_c = pad16(2 * std::max(b->nc, 1));
    // log(2 pi sigma2) over the fine pixels (storeWeightedSums :9032-9038)
    b->logsigma2 = 0.;
    for (const PixelRef &p : b->pf_h)
        if (p.shell > 0 && p.shell < d.sigma2_len) b->logsigma2 += std::log(2. * kPi * b->sigma2[p.shell]);
    GBR_CUDA(b->pc.upload(b->pc_h.data(), b->pc_h.size()));
    GBR_CUDA(b->pf.upload(b->pf_h.data(), b->pf_h.size()));
    GBR_CUDA(b->minv_c.upload(mc.data(), mc.size()));
    GBR_CUDA(b->minv_f.upload(mf.data(), mf.size()));
    GBR_CUDA(b->minv_store.upload(ms.data(), ms.size()));

    // ---- orientation tables ----
    const long R = b->R, RF = b->RF;
    std::vector<float> ec((size_t)R * 9), ef((size_t)RF * 9), po(R);
    std::vector<int> cc(R), cf(RF), cr(R);
    double mean = 0.;
    for (long ic = 0; ic < b->K; ++ic)
        for (long id = 0; id < b->ND; ++id)
            for (long is = 0; is < b->NP; ++is) mean += b->pdf_dir[ic * b->ND + id];
    mean /= (double)R;
    std::vector<double> fr(b->nOR), ft(b->nOR), fp(b->nOR);
    double A[9], Ai[9];
    // r_max-circle pixels of the coarse / fine lists (projector geometry) and
    // of the fine list (backprojector geometry)
    std::vector<int> pcc, pcf, bcf;
    const long pr2 = (long)b->pg.r_max * b->pg.pad * b->pg.r_max * b->pg.pad;
    const long brr = iround((double)b->bg.r_max * b->bg.pad);
    const long br2 = brr * brr;
    b->use_circ = !b->is2d;
    const int nbc = circle_bits(b->pc_h, b->pg.pad, pr2, pcc), nbf = circle_bits(b->pf_h, b->pg.pad, pr2, pcf),
              nbb = circle_bits(b->pf_h, b->bg.pad, br2, bcf);
    if (b->use_circ && (nbc > 64 || nbf > 64 || nbb > 64))
        return fail(GBR_ERR_UNSUPPORTED, "more than 64 pixels on the r_max circle");
    const std::vector<int> onc = circle_pixels(pcc), onf = circle_pixels(pcf), onb = circle_pixels(bcf);
    std::vector<unsigned long long> pmc(b->use_circ ? R : 0), pmf(b->use_circ ? RF : 0), bmf(b->use_circ ? RF : 0);
    const int shf = b->cur / 2 + 1;
    for (long ic = 0; ic < b->K; ++ic)
        for (long id = 0; id < b->ND; ++id)
            for (long is = 0; is < b->NP; ++is) {
                const long r = (ic * b->ND + id) * b->NP + is;
                euler_to_matrix(b->grid.dir_rot[id], b->grid.dir_tilt[id], b->grid.psi[is], A);
                for (int a = 0; a < 3; ++a)
                    for (int c = 0; c < 3; ++c) ec[(size_t)r * 9 + a * 3 + c] = (float)(A[c * 3 + a] * d.padding_factor);
                if (b->use_circ && nbc) {
                    ref_inverse_pad(A, (double)b->pg.pad, Ai);
                    pmc[r] = circle_mask(b->pc_h, onc, pcc, Ai, false, (int)pr2, 0);
                }
                double pdf = b->pdf_dir[ic * b->ND + id];
                if (mean != 0.) pdf /= mean;
                po[r] = (b->pdf_class[ic] > 0. && b->pdf_dir[ic * b->ND + id] > 0.) ? (float)pdf : 0.f;
                cc[r] = (int)ic;
                cr[r] = (int)ic;
                b->grid.fine_orientations(id, is, fr.data(), ft.data(), fp.data());
                for (long io = 0; io < b->nOR; ++io) {
                    const long rf = r * b->nOR + io;
                    euler_to_matrix(fr[io], ft[io], fp[io], A);
                    for (int a = 0; a < 3; ++a)
                        for (int c = 0; c < 3; ++c)
                            ef[(size_t)rf * 9 + a * 3 + c] = (float)(A[c * 3 + a] * d.padding_factor);
                    if (b->use_circ && (nbf || nbb)) {
                        ref_inverse_pad(A, (double)b->pg.pad, Ai);
                        if (nbf) pmf[rf] = circle_mask(b->pf_h, onf, pcf, Ai, false, (int)pr2, 0);
                        if (b->bg.pad != b->pg.pad) ref_inverse_pad(A, (double)b->bg.pad, Ai);
                        if (nbb) bmf[rf] = circle_mask(b->pf_h, onb, bcf, Ai, true, (int)br2, shf);
                    }
                    cf[rf] = (int)ic;
                }
            }
    GBR_CUDA(b->eul_c.upload(ec.data(), ec.size()));
    GBR_CUDA(b->eul_f.upload(ef.data(), ef.size()));
    GBR_CUDA(b->cls_c.upload(cc.data(), cc.size()));
    GBR_CUDA(b->cls_f.upload(cf.data(), cf.size()));
    GBR_CUDA(b->cls_of_r.upload(cr.data(), cr.size()));
    GBR_CUDA(b->pdf_orient.upload(po.data(), po.size()));
    if (b->use_circ) {
        GBR_CUDA(b->pcirc_c.upload(pcc.data(), pcc.size()));
        GBR_CUDA(b->pcirc_f.upload(pcf.data(), pcf.size()));
        GBR_CUDA(b->bcirc_f.upload(bcf.data(), bcf.size()));
        GBR_CUDA(b->pmask_c.upload(pmc.data(), pmc.size()));
        GBR_CUDA(b->pmask_f.upload(pmf.data(), pmf.size()));
        GBR_CUDA(b->bmask_f.upload(bmf.data(), bmf.size()));
    }
    b->pdf_orient_min = 0.f;
    b->pdf_orient_max = 0.f;
    for (float v : po) {
        if (v > 0.f && (b->pdf_orient_min == 0.f || v < b->pdf_orient_min)) b->pdf_orient_min = v;
        b->pdf_orient_max = std::max(b->pdf_orient_max, v);
    }

    // ---- translations and phase tables ----
    std::vector<double> tx(b->grid.trans_x), ty(b->grid.trans_y);
    std::vector<double> ctx(b->T), cty(b->T);
    for (long t = 0; t < b->T; ++t) {
        ctx[t] = tx[t] / pix;
        cty[t] = ty[t] / pix;
    }
    b->otx_h.assign(b->TF, 0.);
    b->oty_h.assign(b->TF, 0.);
    for (long t = 0; t < b->T; ++t) b->grid.fine_translations(t, pix, &b->otx_h[t * b->nOT], &b->oty_h[t * b->nOT]);
    GBR_CUDA(b->tx.upload(tx.data(), tx.size()));
    GBR_CUDA(b->ty.upload(ty.data(), ty.size()));
    GBR_CUDA(b->otx.upload(b->otx_h.data(), b->otx_h.size()));
    GBR_CUDA(b->oty.upload(b->oty_h.data(), b->oty_h.size()));
    DevBuf<double> ctx_d, cty_d;
    GBR_CUDA(ctx_d.upload(ctx.data(), ctx.size()));
    GBR_CUDA(cty_d.upload(cty.data(), cty.size()));
    GBR_CUDA(b->phase_c.reserve((size_t)b->T * b->ldk_c));
    GBR_CUDA(b->phase_c.zero());
    GBR_CUDA(launch_phase_table(b->phase_c.p, ctx_d.p, cty_d.p, (int)b->T, b->pc.p, b->nc, b->ldk_c,
                                (double)d.ori_size, 0));
    GBR_CUDA(b->phase_f.reserve((size_t)b->TF * b->nf));
    GBR_CUDA(launch_phase_table(b->phase_f.p, b->otx.p, b->oty.p, (int)b->TF, b->pf.p, b->nf, b->nf,
                                (double)d.ori_size, 0));

    // ---- coarse projections (shared by every batch of the iteration) ----
    std::vector<const float2 *> vp(b->K);
    for (long k = 0; k < b->K; ++k) vp[k] = b->vol[k].p;
    GBR_CUDA(b->vols_d.upload(vp.data(), vp.size()));
    const unsigned long long *texs = nullptr;
    if (!b->is2d) {
        b->vtex.resize(b->K);
        std::vector<unsigned long long> th(b->K);
        for (long k = 0; k < b->K; ++k) {
            GBR_CUDA(gbr::vol_texture_update(b->vtex[k], b->vol[k].p, b->pg, 0));
            th[k] = (unsigned long long)b->vtex[k].tex;
        }
        GBR_CUDA(b->texs_d.upload(th.data(), th.size()));
        texs = b->texs_d.p;
    }
    GBR_CUDA(b->proj_c.reserve((size_t)R * b->lda_c));
    GBR_CUDA(b->proj2_c.reserve((size_t)R * b->ldk_c));
    GBR_CUDA(b->proj_c.zero());
    GBR_CUDA(b->proj2_c.zero());
    GBR_CUDA(launch_project_rows(b->vols_d.p, b->pg, b->eul_c.p, b->cls_c.p, nullptr, (int)R, b->pc.p, b->nc,
                                 b->proj_c.p, b->lda_c, b->proj2_c.p, b->ldk_c, nullptr, 0,
                                 b->use_circ ? b->pcirc_c.p : nullptr, b->use_circ ? b->pmask_c.p : nullptr,
                                 (b->crs / 2) * (b->crs / 2), texs));
    if (d.precision == GBR_PREC_BF16) {
        GBR_CUDA(b->proj_c_tc.reserve(tc_a_bytes((int)R, 2 * b->nc)));
        GBR_CUDA(launch_tc_pack_a(b->proj_c.p, b->lda_c, (int)R, 2 * b->nc, b->proj_c_tc.p, 0));
        GBR_CUDA(b->proj2_c_tf.reserve(tc_norm_a_bytes((int)R, b->nc)));
        GBR_CUDA(launch_tc_norm_pack_a(b->proj2_c.p, b->ldk_c, (int)R, b->nc, b->proj2_c_tf.p, 0));
        int flag = 0;
        GBR_CUDA(tc_error_flag(&flag, 1));
    }
    // ---- fine projections of every oversampled orientation ----
    b->ldk_f = pad16(std::max(b->nf, 1));
    b->lda_f = 2 * b->ldk_f;
    GBR_CUDA(b->proj_f.reserve((size_t)RF * b->lda_f));
    GBR_CUDA(b->proj2_f.reserve((size_t)RF * b->ldk_f));
    GBR_CUDA(b->proj_f.zero());
    GBR_CUDA(b->proj2_f.zero());
    GBR_CUDA(launch_project_rows(b->vols_d.p, b->pg, b->eul_f.p, b->cls_f.p, nullptr, (int)RF, b->pf.p, b->nf,
                                 b->proj_f.p, b->lda_f, b->proj2_f.p, b->ldk_f, nullptr, 0,
                                 b->use_circ ? b->pcirc_f.p : nullptr, b->use_circ ? b->pmask_f.p : nullptr,
                                 (b->cur / 2) * (b->cur / 2), texs));
    // ---- slice accumulators ----
    GBR_CUDA(b->bpimg.reserve((size_t)RF * b->nf));
    GBR_CUDA(b->bpw.reserve((size_t)RF * b->nf));
    GBR_CUDA(b->active.reserve(RF));
    GBR_CUDA(b->bpimg.zero());
    GBR_CUDA(b->bpw.zero());
    GBR_CUDA(b->active.zero());
    // scale-correction shell mask data_vs_prior > 3
    std::vector<unsigned char> dm((size_t)b->K * b->nshell, 0);
    if (d.do_scale_correction && !b->dvp.empty())
        for (size_t i = 0; i < dm.size(); ++i) dm[i] = b->dvp[i] > 3. ? 1 : 0;
    GBR_CUDA(b->dvp_mask.upload(dm.data(), dm.size()));
    GBR_CUDA(cudaDeviceSynchronize());
    b->tables_ready = true;
    return GBR_OK;
}

int ensure_capacity(gbr_worker *w, int n) {
    gbr_bundle *b = w->b;
    if (n <= w->cap) return GBR_OK;
    ++w->buf_gen;
    w->masks_clean = false;
    const size_t full = (size_t)b->full_npix;
    GBR_CUDA(w->X.reserve(n * full));
    GBR_CUDA(w->Xn.reserve(n * full));
    GBR_CUDA(w->C.reserve(n * full));
    GBR_CUDA(w->pdat.reserve((size_t)n * 8));
    GBR_CUDA(w->power.reserve((size_t)n * b->nshell));
    GBR_CUDA(w->a_c.reserve((size_t)n * b->ldk_c));
    GBR_CUDA(w->b_c.reserve((size_t)n * b->ldk_c));
    GBR_CUDA(w->a_f.reserve((size_t)n * b->ldk_f));
    GBR_CUDA(w->b_f.reserve((size_t)n * b->ldk_f));
    GBR_CUDA(w->Xf.reserve((size_t)n * b->nf));
    GBR_CUDA(w->Xnf.reserve((size_t)n * b->nf));
    GBR_CUDA(w->Cf.reserve((size_t)n * b->nf));
    GBR_CUDA(w->ps.reserve(n));
    GBR_CUDA(w->pdf_off.reserve((size_t)n * b->KP * b->T));
    GBR_CUDA(w->nrm.reserve((size_t)n * b->R));
    GBR_CUDA(w->vals.reserve((size_t)n * b->R * b->T));
    GBR_CUDA(w->seg_c.reserve(n + 1));
    GBR_CUDA(w->seg_f.reserve(n + 1));
    GBR_CUDA(w->hist.reserve((size_t)n * kHistBins));
    const int W = (int)((b->T + 31) / 32);
    GBR_CUDA(w->mask.reserve((size_t)n * b->R * W));
    GBR_CUDA(w->cnt.reserve((size_t)n * b->R));
    GBR_CUDA(w->scan_tmp.reserve(2 * (size_t)fine_jobs_nblocks((long long)n * b->R) + 2));
    GBR_CUDA(w->jobs.reserve((size_t)n * b->R));
    GBR_CUDA(w->need_r.reserve(b->R));
    GBR_CUDA(w->shell.reserve((size_t)n * b->nshell));
    GBR_CUDA(w->pacc.reserve((size_t)n * 8));
    GBR_CUDA(w->hist.zero());
    std::vector<long long> seg(n + 1);
    for (int p = 0; p <= n; ++p) seg[p] = (long long)p * b->R * b->T;
    GBR_CUDA(w->seg_c.upload(seg.data(), seg.size()));
    w->cap = n;
    return GBR_OK;
}

// Worker buffers for a call of n_all particles: the tables of the bundle and
// the batch capacity (particles per pass, bounded by the device budget).
int call_capacity(gbr_worker *w, int n_all) {
    gbr_bundle *b = w->b;
    int s = build_tables(b);
    if (s) return s;
    // device bytes per particle of the coarse pass (the dense fine pass is
    // only chosen when its array also fits, see run_batch)
    const long long per_part = (long long)b->R * b->T * 4 + (1LL << 20);
    const long long mem_cap = (b->budget ? (long long)b->budget : (48LL << 30)) / 2;
    int cap = (int)std::max<long long>(1, std::min<long long>(1024, mem_cap / per_part));
    if (w->batch_cap > 0) cap = std::min(cap, w->batch_cap);
    if (w->debug) {
        w->dbg.clear();
        w->dbg_n = 0;
    }
    s = ensure_capacity(w, std::min(cap, n_all));
    if (s) return s;
    // passes of this call: at most `cap` particles each (the buffers may hold more)
    w->pass_cap = std::min(cap, n_all);
    return GBR_OK;
}

int threshold_search(gbr_worker *w, int n, float *vals, const long long *seg, long long max_len, int coarse,
                     const long long *seg_end = nullptr, long long n_total = 0) {
    gbr_bundle *b = w->b;
    const double f = b->d.adaptive_fraction;
    const int pass = coarse ? 1 : 2;
    if (max_len <= kSelectFusedMax) {
        w->launches += 1;
        GBR_CUDA(launch_select_fused(vals, seg, seg_end, n, n_total, pass, f, coarse, w->ps.p, w->st));
        return GBR_OK;
    }
    w->launches += 6;
    GBR_CUDA(launch_hist_refine(vals, seg, n, max_len, 0, w->ps.p, w->hist.p, w->st, pass, f, seg_end, n_total));
    GBR_CUDA(launch_select(n, 0, f, coarse, w->ps.p, w->hist.p, w->st));
    GBR_CUDA(launch_hist_refine(vals, seg, n, max_len, 1, w->ps.p, w->hist.p, w->st, pass, f, seg_end, n_total));
    GBR_CUDA(launch_select(n, 1, f, coarse, w->ps.p, w->hist.p, w->st));
    GBR_CUDA(launch_hist_refine(vals, seg, n, max_len, 2, w->ps.p, w->hist.p, w->st, pass, f, seg_end, n_total));
    GBR_CUDA(launch_select(n, 2, f, coarse, w->ps.p, w->hist.p, w->st));
    return GBR_OK;
}

// Fine pass over sparse jobs (few significant coarse poses): one block per
// (particle, significant coarse orientation), weighted sums by atomics.
int fine_sparse(gbr_worker *w, int n, long long njobs, long long nfine, const std::vector<long long> &segf,
                long long &max_seg) {
    gbr_bundle *b = w->b;
    cudaStream_t st = w->st;
    const int R = (int)b->R, T = (int)b->T, nOR = (int)b->nOR, nOT = (int)b->nOT, W = (T + 31) / 32;
    max_seg = 0;
    for (int p = 0; p < n; ++p) max_seg = std::max(max_seg, segf[p + 1] - segf[p]);
    GBR_CUDA(w->fd.reserve(nfine));
    GBR_CUDA(w->ejob.reserve(nfine));
    GBR_CUDA(w->ecode.reserve(nfine));
    GBR_CUDA(cudaEventRecord(w->ev[5], st));
    const float2 *projf = reinterpret_cast<const float2 *>(b->proj_f.p);
    // work queue of (job, pixel range) items; the job count is read on the device
    const int nsplit = fine_diff2_nsplit(b->nf);
    GBR_CUDA(w->fq_part.reserve((size_t)nfine * nsplit));
    GBR_CUDA(w->fq_npart.reserve((size_t)njobs * 8 * nsplit));
    GBR_CUDA(w->fq_arrive.reserve(njobs));
    GBR_CUDA(w->fq_head.reserve(1));
    GBR_CUDA(launch_fine_diff2(w->jobs.p, w->scan_tmp.p + 2 * fine_jobs_nblocks((long long)n * R), njobs, nsplit,
                               w->fq_head.p, w->fq_arrive.p, w->fq_part.p, w->fq_npart.p, w->mask.p, R, T, W, nOR,
                               nOT, projf, b->ldk_f, w->b_f.p, w->a_f.p, b->nf, b->phase_f.p, w->fd.p, w->ejob.p,
                               w->ecode.p, w->ps.p, st));
    GBR_CUDA(cudaEventRecord(w->ev[6], st));
    if (w->debug) {
        gbr_worker::DbgPass &D = w->dbg.back();
        D.fine.resize(nfine);
        D.ejob.resize(nfine);
        D.ecode.resize(nfine);
        D.jobs.resize(njobs);
        GBR_CUDA(cudaMemcpyAsync(D.fine.data(), w->fd.p, sizeof(float) * nfine, cudaMemcpyDeviceToHost, st));
        GBR_CUDA(cudaMemcpyAsync(D.ejob.data(), w->ejob.p, sizeof(int) * nfine, cudaMemcpyDeviceToHost, st));
        GBR_CUDA(cudaMemcpyAsync(D.ecode.data(), w->ecode.p, sizeof(unsigned) * nfine, cudaMemcpyDeviceToHost, st));
        GBR_CUDA(cudaMemcpyAsync(D.jobs.data(), w->jobs.p, sizeof(FineJob) * njobs, cudaMemcpyDeviceToHost, st));
        D.segf = segf;
    }
    GBR_CUDA(launch_weights(w->fd.p, w->seg_f.p, n, max_seg, 0, T, w->ejob.p, w->ecode.p, w->jobs.p, nOR, nOT,
                            b->pdf_orient.p, w->pdf_off.p, w->ps.p, w->hist.p, st, 1, b->KP, (int)(b->ND * b->NP)));
    int s = threshold_search(w, n, w->fd.p, w->seg_f.p, max_seg, 0);
    if (s) return s;
    GBR_CUDA(cudaEventRecord(w->ev[7], st));
    if (w->debug) {
        gbr_worker::DbgPass &D = w->dbg.back();
        D.wfine.resize(nfine);
        GBR_CUDA(cudaMemcpyAsync(D.wfine.data(), w->fd.p, sizeof(float) * nfine, cudaMemcpyDeviceToHost, st));
    }
    WsumArgs wa{};
    wa.jobs = w->jobs.p;
    wa.njobs = njobs;
    wa.mask = w->mask.p;
    wa.R = R; wa.T = T; wa.W = W; wa.nOR = nOR; wa.nOT = nOT; wa.nf = b->nf; wa.ldpf = b->ldk_f;
    wa.nshell = b->nshell; wa.ndir = (int)b->ND; wa.npsi = (int)b->NP; wa.K = (int)b->K;
    wa.w = w->fd.p;
    wa.ps = w->ps.p;
    wa.projf = projf;
    wa.Xf = w->Xf.p; wa.Xnf = w->Xnf.p; wa.Cf = w->Cf.p;
    wa.minv_store = b->minv_store.p;
    wa.pf = b->pf.p;
    wa.phase_f = b->phase_f.p;
    wa.otx = b->otx.p; wa.oty = b->oty.p;
    wa.pdat = w->pdat.p;
    wa.pixel = b->d.pixel_size;
    wa.do_scale = (int)b->d.do_scale_correction;
    wa.dvp_mask = b->dvp_mask.p;
    wa.bpimg = b->bpimg.p; wa.bpw = b->bpw.p; wa.active = b->active.p;
    wa.shell = w->shell.p; wa.pacc = w->pacc.p;
    wa.pdf_dir = b->w_pdf_dir.p; wa.pdf_cls = b->w_pdf_cls.p;
    wa.class_prior = b->is2d ? b->class_prior.p : nullptr;
    wa.w_prior_off = b->is2d ? b->w_prior_off.p : nullptr;
    // direct insertion of each job's weighted slices into the staging volumes
    wa.bp_direct = w->bp_direct;
    wa.eul_f = b->eul_f.p;
    wa.stage = b->bps_ptrs.p;
    wa.bg = b->bg;
    wa.circ = b->use_circ ? b->bcirc_f.p : nullptr;
    wa.cmask = b->use_circ ? b->bmask_f.p : nullptr;
    w->last_direct = w->bp_direct;
    GBR_CUDA(launch_wsum(wa, st));
    w->launches += 3;
    return GBR_OK;
}

// Fine pass over every oversampled pose (most coarse poses significant):
// fine diff2 and the weighted sums as dense contractions.
int fine_dense(gbr_worker *w, int n, long long &seg_len) {
    gbr_bundle *b = w->b;
    cudaStream_t st = w->st;
    const int R = (int)b->R, T = (int)b->T, nOR = (int)b->nOR, nOT = (int)b->nOT, W = (T + 31) / 32;
    const int RF = (int)b->RF, TF = (int)b->TF, nf = b->nf;
    const long long per = (long long)RF * TF;
    seg_len = per;
    GBR_CUDA(w->fd.reserve((size_t)n * per));
    GBR_CUDA(w->fnrm.reserve((size_t)n * RF));
    std::vector<long long> seg(n + 1);
    for (int p = 0; p <= n; ++p) seg[p] = (long long)p * per;
    GBR_CUDA(cudaMemcpyAsync(w->seg_f.p, seg.data(), sizeof(long long) * (n + 1), cudaMemcpyHostToDevice, st));
    GBR_CUDA(cudaEventRecord(w->ev[5], st));
    // fine norm term N_f[p][rf] and masked dense diff2 [p][rf][tf]
    GBR_CUDA(launch_gemm_rows(b->proj2_f.p, b->ldk_f, RF, w->a_f.p, b->ldk_f, n, b->ldk_f, w->fnrm.p, RF, 1, st));
    GBR_CUDA(launch_gemm_diff2(b->proj_f.p, b->lda_f, RF, 2 * nf, w->b_f.p, b->ldk_f, b->phase_f.p, nf, n, TF,
                               w->fd.p, w->fnrm.p, b->pdf_orient.p, w->mask.p, nOR, nOT, W, w->ps.p, 1, st));
    GBR_CUDA(cudaEventRecord(w->ev[6], st));
    if (w->debug) {
        gbr_worker::DbgPass &D = w->dbg.back();
        D.fine.resize((size_t)n * per);
        GBR_CUDA(cudaMemcpyAsync(D.fine.data(), w->fd.p, sizeof(float) * n * per, cudaMemcpyDeviceToHost, st));
        D.segf = seg;
    }
    GBR_CUDA(launch_weights(w->fd.p, w->seg_f.p, n, per, 2, T, nullptr, nullptr, nullptr, nOR, nOT,
                            b->pdf_orient.p, w->pdf_off.p, w->ps.p, w->hist.p, st, 1, b->KP, (int)(b->ND * b->NP)));
    int s = threshold_search(w, n, w->fd.p, w->seg_f.p, per, 0);
    if (s) return s;
    GBR_CUDA(cudaEventRecord(w->ev[7], st));
    if (w->debug) {
        gbr_worker::DbgPass &D = w->dbg.back();
        D.wfine.resize((size_t)n * per);
        GBR_CUDA(cudaMemcpyAsync(D.wfine.data(), w->fd.p, sizeof(float) * n * per, cudaMemcpyDeviceToHost, st));
    }
    // normalised weights, row sums, scalar sums
    const int ldwt = pad16(n);
    const long long ldz = pad16(n * TF);
    GBR_CUDA(w->Wt.reserve((size_t)RF * ldwt));
    const int ldwp = pad16(RF);
    GBR_CUDA(w->Wp.reserve((size_t)n * ldwp));
    GBR_CUDA(cudaMemsetAsync(w->Wp.p, 0, sizeof(float) * n * ldwp, st));
    GBR_CUDA(w->Zt.reserve((size_t)2 * nf * ldz));
    GBR_CUDA(w->CM.reserve((size_t)nf * ldwt));
    GBR_CUDA(w->G.reserve((size_t)n * nf));
    GBR_CUDA(w->S2P.reserve((size_t)n * nf));
    GBR_CUDA(cudaMemsetAsync(w->Wt.p, 0, sizeof(float) * RF * ldwt, st));
    GBR_CUDA(cudaMemsetAsync(w->G.p, 0, sizeof(float2) * n * nf, st));
    GBR_CUDA(launch_fine_normalize(w->fd.p, n, R, nOR, nOT, T, w->ps.p, w->pdat.p, b->otx.p, b->oty.p,
                                   b->d.pixel_size, (int)b->ND, (int)b->NP, w->Wt.p, ldwt, w->Wp.p, ldwp, b->active.p,
                                   w->pacc.p, b->w_pdf_dir.p, b->w_pdf_cls.p,
                                   b->is2d ? b->class_prior.p : nullptr, b->is2d ? b->w_prior_off.p : nullptr, st));
    // BP slices and weights (batch-summed), sigma2 contractions (per particle)
    GBR_CUDA(launch_make_zt(w->Cf.p, w->Xnf.p, b->minv_store.p, b->phase_f.p, w->pdat.p,
                            (int)b->d.do_scale_correction, n, TF, nf, w->Zt.p, ldz, w->CM.p, ldwt, st));
    GBR_CUDA(launch_gemm_bpimg(w->fd.p, RF, TF, n, w->Zt.p, ldz, 2 * nf, reinterpret_cast<float *>(b->bpimg.p),
                               2 * nf, st));
    GBR_CUDA(launch_gemm_rows(w->Wt.p, ldwt, RF, w->CM.p, ldwt, nf, ldwt, b->bpw.p, nf, 0, st));
    GBR_CUDA(launch_gemm_sigma_cross(w->fd.p, RF, TF, n, b->proj_f.p, b->lda_f, nf, b->phase_f.p, w->G.p, st));
    GBR_CUDA(launch_gemm_sigma_norm(w->Wp.p, ldwp, n, RF, b->proj2_f.p, b->ldk_f, nf, w->S2P.p, st));
    GBR_CUDA(launch_shell_dense(n, w->S2P.p, w->G.p, w->Xf.p, w->Cf.p, b->pf.p, nf, b->nshell, w->pdat.p,
                                (int)b->d.do_scale_correction, b->dvp_mask.p, (int)b->K, w->pacc.p, w->shell.p, st));
    w->launches += 11;
    return GBR_OK;
}

// Orientation blocks of the restricted coarse pass: four sibling HEALPix
// directions (one parent pixel in NEST order) with every psi angle, i.e.
// NB = 4 npsi consecutive rows of the projection table.
constexpr int kDirsPerBlock = 4;

int restricted_supported(const gbr_bundle *b) {
    if (b->d.precision != GBR_PREC_BF16)
        return fail(GBR_ERR_UNSUPPORTED, "restricted coarse pass needs the precision form (tcgen05)");
    if (b->is2d || b->ND % kDirsPerBlock != 0)
        return fail(GBR_ERR_UNSUPPORTED, "restricted coarse pass needs a 3D HEALPix grid of order >= 1");
    const long NB = kDirsPerBlock * b->NP;
    if (NB % 32 != 0 || NB > 256)
        return fail(GBR_ERR_UNSUPPORTED, "restricted coarse pass needs 4 x psi samples = a multiple of 32, <= 256");
    if (b->T > 128) return fail(GBR_ERR_UNSUPPORTED, "restricted coarse pass needs at most 128 translations");
    return GBR_OK;
}

// The coarse cross term of the pass's particles over their own blocks: one
// (particle, block) work item per block a particle scores, in chunks of 64
// particles and block-major inside a chunk (a block's tiles are read from HBM
// once per chunk, the chunk's particle tiles stay in L2).
int restricted_coarse(gbr_worker *w, int n, unsigned int *segmask) {
    gbr_bundle *b = w->b;
    const int R = (int)b->R, T = (int)b->T, NB = kDirsPerBlock * (int)b->NP;
    const int nblk = R / NB;
    const int K2 = 2 * b->nc;
    if (!b->blk_ready) {
        GBR_CUDA(b->proj_c_blk.reserve(tc_blocks_bytes(R, K2, NB)));
        GBR_CUDA(launch_tc_pack_blocks(b->proj_c.p, b->lda_c, R, K2, NB, b->proj_c_blk.p, w->st));
        b->blk_ready = true;
        w->launches += 1;
    }
    std::vector<std::vector<int>> by_block(nblk);
    std::vector<char> seen(nblk);
    GBR_CUDA(w->items_h.reserve((size_t)n * nblk));
    long long ni = 0;
    for (int c0 = 0; c0 < n; c0 += 64) {
        const int c1 = std::min(n, c0 + 64);
        for (auto &v : by_block) v.clear();
        for (int p = c0; p < c1; ++p) {
            const int32_t *row = w->restrict_blocks + (size_t)(w->pass_p0 + p) * w->restrict_m;
            if (w->restrict_m > 0 && row[0] == GBR_ALL_BLOCKS) {
                for (int o = 0; o < nblk; ++o) by_block[o].push_back(p);
                continue;
            }
            std::fill(seen.begin(), seen.end(), 0);
            for (int64_t j = 0; j < w->restrict_m; ++j) {
                const int32_t o = row[j];
                if (o < 0) continue;
                if (o >= nblk) return fail(GBR_ERR_INVALID, "orientation block " + std::to_string(o) +
                                                                " out of range (" + std::to_string(nblk) + " blocks)");
                if (!seen[o]) {
                    seen[o] = 1;
                    by_block[o].push_back(p);
                }
            }
        }
        for (int o = 0; o < nblk; ++o)
            for (int p : by_block[o]) w->items_h.p[ni++] = make_int2(p, o);
    }
    w->last_items = ni;
    if (ni == 0) return fail(GBR_ERR_NUMERICAL, "no orientation block to score in this batch");
    GBR_CUDA(w->items_d.reserve(ni));
    GBR_CUDA(cudaMemcpyAsync(w->items_d.p, w->items_h.p, sizeof(int2) * ni, cudaMemcpyHostToDevice, w->st));
    GBR_CUDA(w->ytp.reserve(tc_yp_bytes(n, K2)));
    GBR_CUDA(launch_tc_blocks(b->proj_c_blk.p, NB, w->ytp.p, R, K2, w->b_c.p, b->ldk_c, b->phase_c.p, b->ldk_c, n, T,
                              w->items_d.p, (int)ni, w->vals.p, w->nrm.p, b->pdf_orient.p, w->ps.p, w->rowmin.p,
                              segmask, w->st));
    w->launches += 2;  // particle tiles + tensor-core kernel
    return GBR_OK;
}

// One sub-batch of n <= cap particles whose inputs are already in w->X etc.
// Adds the staged insertions of every class into the FP64 volumes (after
// all work queued on the device), before the volumes are read or replaced.
int flush_staged(gbr_bundle *b) {
    GBR_CUDA(cudaDeviceSynchronize());
    if (b->staged == 0) return GBR_OK;
    for (long k = 0; k < b->K; ++k)
        GBR_CUDA(launch_bp_flush(b->bp_stage[k].p, b->bp_data[k].p, b->bp_weight[k].p, b->bg, 0));
    GBR_CUDA(cudaDeviceSynchronize());
    b->staged = 0;
    return GBR_OK;
}

// Host-side choices of a coarse pass (no device work): the restricted form,
// row skip, sparse diff2 writes, the candidate-list capacity.
struct CoarseFlags {
    bool restricted = false, use_rowmin = false, sparse = false;
    int cap = 0;
    long long nbj = 0;
};

CoarseFlags coarse_flags(gbr_worker *w, int n) {
    gbr_bundle *b = w->b;
    const gbr_model_desc &d = b->d;
    const int R = (int)b->R, T = (int)b->T;
    const long long RT = (long long)R * T;
    CoarseFlags cf;
    // a pass whose particles all fall back to the exhaustive search runs the
    // exhaustive kernel (no work-item list)
    cf.restricted = w->restrict_blocks != nullptr;
    if (cf.restricted) {
        bool all = true;
        for (int p = 0; p < n && all; ++p)
            all = w->restrict_blocks[(size_t)(w->pass_p0 + p) * w->restrict_m] == GBR_ALL_BLOCKS;
        if (all) cf.restricted = false;
        w->last_items = all ? (long long)n * (R / (kDirsPerBlock * (int)b->NP)) : 0;
    }
    cf.use_rowmin = d.precision == GBR_PREC_BF16 && (cf.restricted || (T >= 32 && w->coarse_rows == 0));
    // sparse diff2 writes: only row segments near the running minimum are
    // stored (the debug read-back reports the others as not computed); the
    // restricted pass stores the rows of the blocks it scores
    cf.sparse = cf.use_rowmin && (cf.restricted || T <= 960);
    cf.cap = (int)std::min<long long>(RT, w->cand_cap_max);
    cf.nbj = fine_jobs_nblocks((long long)n * R);
    return cf;
}

// Event record that stream capture turns into an event node of the graph,
// so that the stage times stay measurable when the graph is replayed.
cudaError_t record(cudaEvent_t ev, cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess) return e;
    return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal)
                                               : cudaEventRecord(ev, st);
}

// Fine-pass job lists from the significance counts, and their read-back
// (with the tensor-core pipeline's error flag on the first try).
int jobs_readback(gbr_worker *w, int n, long long nbj, bool tc_check) {
    gbr_bundle *b = w->b;
    cudaStream_t st = w->st;
    const int R = (int)b->R;
    GBR_CUDA(record(w->ev[4], st));
    GBR_CUDA(cudaMemsetAsync(w->need_r.p, 0, R, st));
    GBR_CUDA(launch_fine_jobs(w->cnt.p, n, R, (int)(b->nOR * b->nOT), w->scan_tmp.p, w->jobs.p, w->seg_f.p,
                              w->need_r.p, st));
    GBR_CUDA(cudaMemcpyAsync(w->h_totals.p, w->scan_tmp.p + 2 * nbj, sizeof(long long) * 2, cudaMemcpyDeviceToHost,
                             st));
    GBR_CUDA(cudaMemcpyAsync(w->h_segf.p, w->seg_f.p, sizeof(long long) * (n + 1), cudaMemcpyDeviceToHost, st));
    if (tc_check) GBR_CUDA(tc_error_flag_async(w->h_tcflag.p, st));
    w->launches += 3;
    return GBR_OK;
}

// The coarse pass of a batch up to the read-back of its fine job lists:
// preparation, norms, cross term, weights, significance, job lists.  It
// holds no host synchronisation, which makes it the part of a call that is
// captured as a CUDA graph and replayed (run_coarse).
int coarse_segment(gbr_worker *w, int n, const CoarseFlags &cf) {
    gbr_bundle *b = w->b;
    const gbr_model_desc &d = b->d;
    cudaStream_t st = w->st;
    const int R = (int)b->R, T = (int)b->T, nOR = (int)b->nOR, nOT = (int)b->nOT;
    const int W = (T + 31) / 32;
    const long long RT = (long long)R * T;
    GBR_CUDA(record(w->ev[0], st));
    // ---- prep ----
    GBR_CUDA(launch_prep(w->X.p, w->C.p, w->pdat.p, n, b->full_npix, b->pc.p, b->nc, b->minv_c.p, b->ldk_c,
                         b->pf.p, b->nf, b->ldk_f, b->minv_f.p, w->a_c.p, w->b_c.p, w->a_f.p, w->b_f.p, w->Xf.p,
                         w->Xnf.p, w->Cf.p, w->Xn.p, (int)d.do_scale_correction, w->ps.p, st));
    // orientation part of the coarse skip distance: ln(R T) + ln(max/min pdf_orient) + ln(1e10)
    const double log_rt_orient = b->pdf_orient_min > 0.f
                                     ? std::log((double)RT) + std::log((double)b->pdf_orient_max / b->pdf_orient_min) +
                                           std::log(1e10)
                                     : INFINITY;
    GBR_CUDA(launch_pdf_offset(w->pdat.p, n, b->tx.p, b->ty.p, T, d.sigma2_offset, d.pixel_size, w->pdf_off.p,
                               log_rt_orient, w->ps.p, b->KP, b->is2d ? b->class_prior.p : nullptr, st));
    GBR_CUDA(cudaMemsetAsync(w->shell.p, 0, sizeof(double) * n * b->nshell, st));
    GBR_CUDA(cudaMemsetAsync(w->pacc.p, 0, sizeof(double) * n * 8, st));
    GBR_CUDA(record(w->ev[1], st));
    // ---- coarse norm and cross GEMMs ----
    if (d.precision == GBR_PREC_BF16) {
        // tensor cores, TF32 three-term split (FP32-level accuracy)
        GBR_CUDA(w->wtf.reserve(tc_norm_b_bytes(n, b->nc)));
        GBR_CUDA(launch_tc_norm(b->proj2_c_tf.p, w->a_c.p, b->ldk_c, (int)R, b->nc, n, w->wtf.p, w->nrm.p, st));
        w->launches += 4;  // prep, pdf_offset, norm operand packing, norms
    } else {
        GBR_CUDA(launch_gemm_rows(b->proj2_c.p, b->ldk_c, R, w->a_c.p, b->ldk_c, n, b->ldk_c, w->nrm.p, R, 1, st));
        w->launches += 3;  // prep, pdf_offset, norms
    }
    GBR_CUDA(record(w->ev[2], st));
    const bool restricted = cf.restricted, use_rowmin = cf.use_rowmin, sparse = cf.sparse;
    if (w->debug) {
        w->dbg.emplace_back();
        w->dbg.back().n = n;
        w->dbg.back().sparse = sparse ? 1 : 0;
    }
    if (use_rowmin) {
        GBR_CUDA(w->rowmin.reserve((size_t)n * R));
        GBR_CUDA(cudaMemsetAsync(w->rowmin.p, 0xFF, sizeof(unsigned int) * (size_t)n * R, st));
    }
    if (sparse) {
        GBR_CUDA(w->segmask.reserve((size_t)n * R));
        GBR_CUDA(cudaMemsetAsync(w->segmask.p, 0, sizeof(unsigned int) * (size_t)n * R, st));
    }
    unsigned int *segmask = sparse ? w->segmask.p : nullptr;
    if (restricted) {
        int s2 = restricted_coarse(w, n, segmask);
        if (s2) return s2;
    } else if (d.precision == GBR_PREC_BF16) {
        GBR_CUDA(w->ytc.reserve(tc_y_bytes(n * T, 2 * b->nc)));
        GBR_CUDA(launch_tc_diff2(b->proj_c_tc.p, w->ytc.p, R, 2 * b->nc, w->b_c.p, b->ldk_c, b->phase_c.p, b->ldk_c, n,
                                 T, w->vals.p, w->nrm.p, b->pdf_orient.p, w->ps.p,
                                 use_rowmin ? w->rowmin.p : nullptr, segmask, st, w->tc_tune));
        w->launches += 2;  // operand packing + tensor-core kernel
    } else {
        GBR_CUDA(launch_gemm_diff2(b->proj_c.p, b->lda_c, R, 2 * b->nc, w->b_c.p, b->ldk_c, b->phase_c.p, b->ldk_c,
                                   n, T, w->vals.p, w->nrm.p, b->pdf_orient.p, nullptr, 1, 1, W, w->ps.p, 0, st));
        w->launches += 1;
    }
    GBR_CUDA(record(w->ev[3], st));
    if (w->debug) {
        gbr_worker::DbgPass &D = w->dbg.back();
        D.coarse.resize((size_t)n * RT);
        GBR_CUDA(cudaMemcpyAsync(D.coarse.data(), w->vals.p, sizeof(float) * n * RT, cudaMemcpyDeviceToHost, st));
        if (sparse) {
            D.segmask.resize((size_t)n * R);
            GBR_CUDA(cudaMemcpyAsync(D.segmask.data(), w->segmask.p, sizeof(unsigned int) * n * R,
                                     cudaMemcpyDeviceToHost, st));
        }
    }
    // ---- coarse weights and significance ----
    // one read of the diff2 array: weights, FP64 sums and the candidate lists;
    // the threshold search and the significance masks then run on the lists
    const int cap = cf.cap;
    if (w->cand_cap < cap || w->cand_idx.n < (size_t)n * cap) {
        GBR_CUDA(w->cand_idx.reserve((size_t)n * cap));
        GBR_CUDA(w->cand_w.reserve((size_t)n * cap));
        w->cand_cap = cap;
    }
    GBR_CUDA(w->cand_cnt.reserve(n));
    GBR_CUDA(w->cand_seg.reserve(2 * (size_t)n));
    GBR_CUDA(cudaMemsetAsync(w->cand_cnt.p, 0, sizeof(unsigned int) * n, st));
    float *dense_w = nullptr;
    if (w->debug) {
        GBR_CUDA(w->dense_dbg.reserve((size_t)n * RT));
        dense_w = w->dense_dbg.p;
    }
    GBR_CUDA(launch_weights_cand(w->vals.p, n, R, T, b->pdf_orient.p, b->pdf_orient_min, w->pdf_off.p,
                                 d.adaptive_fraction, w->ps.p, w->cand_idx.p, w->cand_w.p, w->cand_cnt.p, cap,
                                 dense_w, use_rowmin ? w->rowmin.p : nullptr, b->KP, (int)(b->ND * b->NP), segmask,
                                 w->cand_buf, st));
    w->launches += 1;
    GBR_CUDA(w->h_ccnt.reserve(n));
    GBR_CUDA(w->h_totals.reserve(2));
    GBR_CUDA(w->h_segf.reserve(n + 1));
    GBR_CUDA(w->h_tcflag.reserve(1));
    // Speculative: the candidate lists are taken as complete and the host
    // checks their counts at the job-list read-back; if one overflowed
    // (flat posterior), the threshold search reruns on the full weight array.
    GBR_CUDA(launch_cand_seg(w->cand_cnt.p, n, cap, w->cand_seg.p, st));
    int s = threshold_search(w, n, w->cand_w.p, w->cand_seg.p, cap, 1, w->cand_seg.p + n, RT);
    if (s) return s;
    // mask and cnt are all zero here (cleared after the previous pass's fine
    // pass, or by run_batch after a reallocation or a failed call)
    GBR_CUDA(launch_cand_masks(w->cand_idx.p, w->cand_w.p, w->cand_cnt.p, cap, n, R, T, W, w->ps.p, w->mask.p,
                               w->cnt.p, st));
    GBR_CUDA(cudaMemcpyAsync(w->h_ccnt.p, w->cand_cnt.p, sizeof(unsigned int) * n, cudaMemcpyDeviceToHost, st));
    w->launches += 2;
    if (w->debug) {
        gbr_worker::DbgPass &D = w->dbg.back();
        D.wcoarse.resize((size_t)n * RT);
        GBR_CUDA(cudaMemcpyAsync(D.wcoarse.data(), dense_w, sizeof(float) * n * RT, cudaMemcpyDeviceToHost, st));
    }
    return jobs_readback(w, n, cf.nbj, d.precision == GBR_PREC_BF16);
}

// Runs coarse_segment directly, or captured as a CUDA graph, or replays the
// captured graph.  A pass of the same batch size as a previous direct pass
// that allocated nothing, with no model, table, option or buffer change
// since (the graph key), is captured; later such passes replay the graph.
// Debug read-backs and the restricted pass (host-built work items) always
// run directly.
int run_coarse(gbr_worker *w, int n, const CoarseFlags &cf) {
    const bool graphable = w->use_graph && !w->debug && !cf.restricted;
    gbr_worker::GraphKey key;
    key.n = n;
    key.api = g_api_gen.load();
    key.buf = w->buf_gen;
    if (graphable && w->gexec && w->g_key == key) {
        GBR_CUDA(cudaGraphLaunch(w->gexec, w->st));
        w->launches += w->g_launches;
        ++w->g_replays;
        return GBR_OK;
    }
    if (!graphable || !(w->warm_key == key)) {
        const unsigned long long a0 = g_alloc_count.load();
        const int s = coarse_segment(w, n, cf);
        if (g_alloc_count.load() != a0) ++w->buf_gen;  // the segment (re)allocated: not yet stable
        w->warm_key = key;
        w->warm_key.buf = w->buf_gen;
        return s;
    }
    // capture: nothing runs until the graph is launched; an allocation in
    // the segment ends the capture with an error (thread-local capture mode)
    const int l0 = w->launches;
    GBR_CUDA(cudaStreamBeginCapture(w->st, cudaStreamCaptureModeThreadLocal));
    const int s = coarse_segment(w, n, cf);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(w->st, &g);
    cudaGraphExec_t ex = nullptr;
    if (s == GBR_OK && e == cudaSuccess && g)
        e = cudaGraphInstantiate(&ex, g, 0);
    else if (e == cudaSuccess)
        e = cudaErrorStreamCaptureInvalidated;
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess || !ex) {
        // not capturable this time: run directly
        (void)cudaGetLastError();
        w->launches = l0;
        w->warm_key = gbr_worker::GraphKey();
        return coarse_segment(w, n, cf);
    }
    if (w->gexec) cudaGraphExecDestroy(w->gexec);
    w->gexec = ex;
    w->g_key = key;
    w->g_launches = w->launches - l0;
    ++w->g_captures;
    GBR_CUDA(cudaGraphLaunch(ex, w->st));
    return GBR_OK;
}

int run_batch(gbr_worker *w, int n, const double *power_h, const double *pdat_h, gbr_particle_result *res) {
    gbr_bundle *b = w->b;
    const gbr_model_desc &d = b->d;
    cudaStream_t st = w->st;
    const int R = (int)b->R, T = (int)b->T, nOR = (int)b->nOR, nOT = (int)b->nOT;
    const int W = (T + 31) / 32;
    const long long RT = (long long)R * T;
    const CoarseFlags cf = coarse_flags(w, n);
    if (!w->masks_clean) {
        // first pass, new buffers or a failed pass: the significance masks and
        // counts start from zero (afterwards each pass clears the rows it used)
        GBR_CUDA(cudaMemsetAsync(w->mask.p, 0, sizeof(unsigned int) * w->mask.n, st));
        GBR_CUDA(cudaMemsetAsync(w->cnt.p, 0, sizeof(int) * w->cnt.n, st));
    }
    w->masks_clean = false;  // until this pass's rows are cleared again
    int s = run_coarse(w, n, cf);
    if (s) return s;
    GBR_CUDA(cudaStreamSynchronize(st));
    if (d.precision == GBR_PREC_BF16 && w->h_tcflag.p[0])
        return fail(GBR_ERR_CUDA, "tensor-core pipeline timed out waiting for its MMAs");
    unsigned int cmax = 0;
    for (int p = 0; p < n; ++p) cmax = std::max(cmax, w->h_ccnt.p[p]);
    if (cmax > (unsigned int)cf.cap) {
        // a candidate list overflowed: significance from the full weight array
        unsigned int *segmask = cf.sparse ? w->segmask.p : nullptr;
        GBR_CUDA(launch_weights(w->vals.p, w->seg_c.p, n, RT, 1, T, nullptr, nullptr, nullptr, nOR, nOT,
                                b->pdf_orient.p, w->pdf_off.p, w->ps.p, w->hist.p, st, 0, b->KP, (int)(b->ND * b->NP),
                                segmask));
        s = threshold_search(w, n, w->vals.p, w->seg_c.p, RT, 1);
        if (s) return s;
        GBR_CUDA(launch_sig_masks(w->vals.p, n, R, T, W, w->ps.p, w->mask.p, w->cnt.p, st));
        w->launches += 2;
        s = jobs_readback(w, n, cf.nbj, false);
        if (s) return s;
        GBR_CUDA(cudaStreamSynchronize(st));
    }
    const long long njobs = w->h_totals.p[0], nfine = w->h_totals.p[1];
    const std::vector<long long> segf(w->h_segf.p, w->h_segf.p + n + 1);
    if (njobs <= 0 || nfine <= 0) return fail(GBR_ERR_NUMERICAL, "no significant coarse samples");
    // ---- fine pass: dense contractions when most poses are significant ----
    const double density = (double)nfine / ((double)n * b->RF * b->TF);
    const long long budget = b->budget ? (long long)b->budget : (48LL << 30);
    const bool dense_fits = (long long)n * b->RF * b->TF * 4 <= budget / 2;
    const bool dense = dense_fits && (w->fine_mode == 1 || (w->fine_mode == 0 && density > 0.1));
    w->last_dense = dense ? 1 : 0;
    long long max_seg = 0;
    if (dense) {
        w->last_direct = 0;  // the dense form fills the slice accumulators
        s = fine_dense(w, n, max_seg);
    } else {
        const long long fine_cap = std::min<long long>(0x7fffffffLL, b->budget ? (long long)b->budget / 24 : (2LL << 30));
        if (nfine > fine_cap)
            return fail(GBR_ERR_OOM, "fine pass needs " + std::to_string(nfine) + " poses in this batch (cap " +
                                         std::to_string(fine_cap) + "); use smaller batches");
        s = fine_sparse(w, n, njobs, nfine, segf, max_seg);
    }
    if (s) return s;
    // the rows this pass set in mask / cnt back to zero for the next pass
    GBR_CUDA(launch_clear_job_rows(w->jobs.p, w->scan_tmp.p + 2 * fine_jobs_nblocks((long long)n * R), njobs, R,
                                   (T + 31) / 32, w->mask.p, w->cnt.p, st));
    w->launches += 1;
    w->masks_clean = true;
    GBR_CUDA(cudaEventRecord(w->ev[8], st));
    // ---- backprojection of the touched slices (already inserted by the
    // weighted sums in the direct form) ----
    if (!w->last_direct) {
        GBR_CUDA(w->act_list.reserve(b->RF));
        GBR_CUDA(w->act_count.reserve(1));
        GBR_CUDA(cudaMemsetAsync(w->act_count.p, 0, sizeof(int), st));
        GBR_CUDA(launch_compact_flags(b->active.p, (int)b->RF, w->act_list.p, w->act_count.p, st));
        GBR_CUDA(launch_backproject(w->act_list.p, w->act_count.p, (int)b->RF, b->eul_f.p, nOR, b->cls_of_r.p,
                                    b->bpimg.p, b->bpw.p, b->pf.p, b->nf, b->bg, b->bps_ptrs.p, b->active.p, st,
                                    b->use_circ ? b->bcirc_f.p : nullptr, b->use_circ ? b->bmask_f.p : nullptr));
        w->launches += 2;
    }
    // the FP32 staging volumes are added into the FP64 volumes once they hold
    // bp_flush particles (and before anything reads the FP64 volumes)
    b->staged += n;
    if (b->staged >= w->bp_flush) {
        for (long k = 0; k < b->K; ++k)
            GBR_CUDA(launch_bp_flush(b->bp_stage[k].p, b->bp_data[k].p, b->bp_weight[k].p, b->bg, st));
        b->staged = 0;
        w->launches += (int)b->K;
    }
    GBR_CUDA(cudaEventRecord(w->ev[9], st));
    // ---- results ----
    GBR_CUDA(w->h_ps.reserve(n));
    GBR_CUDA(w->h_shell.reserve((size_t)n * b->nshell));
    GBR_CUDA(w->h_pacc.reserve((size_t)n * 8));
    const ParticleState *psh = w->h_ps.p;
    const double *shell = w->h_shell.p, *pacc = w->h_pacc.p;
    GBR_CUDA(cudaMemcpyAsync(w->h_ps.p, w->ps.p, sizeof(ParticleState) * n, cudaMemcpyDeviceToHost, st));
    GBR_CUDA(cudaMemcpyAsync(w->h_shell.p, w->shell.p, sizeof(double) * n * b->nshell, cudaMemcpyDeviceToHost, st));
    GBR_CUDA(cudaMemcpyAsync(w->h_pacc.p, w->pacc.p, sizeof(double) * n * 8, cudaMemcpyDeviceToHost, st));
    GBR_CUDA(cudaEventRecord(w->ev[10], st));
    GBR_CUDA(cudaStreamSynchronize(st));
    for (int st_i = 0; st_i < ST_N; ++st_i) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, w->ev[st_i], w->ev[st_i + 1]);
        w->stage_ms[st_i] += ms;
    }
    {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, w->ev_in, w->ev[0]);
        w->stage_ms[ST_N] += ms;
    }
    const auto t_final = std::chrono::steady_clock::now();
    if (w->debug) {
        gbr_worker::DbgPass &D = w->dbg.back();
        D.dense = w->last_dense;
        D.cc.resize(n);
        D.cf.resize(n);
        for (int p = 0; p < n; ++p) {
            D.cc[p] = psh[p].c_coarse;
            D.cf[p] = psh[p].c_fine;
        }
        w->dbg_n += n;
    }
    // ---- per-particle finalisation (storeWeightedSums :8990-9150) ----
    // particles in contiguous ranges over a few host threads; each range
    // adds into its own shell and scalar sums, which are then added in range
    // order
    const int nth = std::max(1, std::min(8, n / 96));
    const int nsh = (int)b->nshell;
    std::vector<double> sig_part((size_t)nth * nsh, 0.);
    struct RangeSums {
        double avg_norm = 0., XA = 0., AA = 0., sumw = 0., off = 0., LL = 0., pmax = 0.;
        int bad = -1;  // first particle with a zero sum of weights
    };
    std::vector<RangeSums> rs(nth);
#pragma omp parallel for num_threads(nth) schedule(static, 1)
    for (int th = 0; th < nth; ++th) {
        const int pa = (int)((long long)n * th / nth), pb = (int)((long long)n * (th + 1) / nth);
        RangeSums &acc = rs[th];
        double *__restrict__ wsig = sig_part.data() + (size_t)th * nsh;
        for (int p = pa; p < pb; ++p) {
            const ParticleState &ps = psh[p];
            gbr_particle_result &o = res[p];
            std::memset(&o, 0, sizeof(o));
            if (!(ps.sum_fine > 0.) || !std::isfinite(ps.sum_fine)) {
                if (acc.bad < 0) acc.bad = p;
                continue;
            }
            const double *pd = pdat_h + (size_t)p * 8;
            o.coarse_min_diff2 = ps.c_coarse + (double)ord2f_host(ps.min_coarse);
            o.coarse_sum_weight = ps.sum_coarse;
            o.coarse_significant_weight = ps.thr_coarse;
            o.fine_min_diff2 = ps.c_fine + (double)ord2f_host(ps.min_fine);
            o.fine_sum_weight = ps.sum_fine;
            o.fine_significant_weight = ps.thr_fine;
            o.nr_sign = ps.nr_sign;
            o.n_fine = segf[p + 1] - segf[p];
            const unsigned long long key = ps.argmax_key;
            const unsigned long long idx = 0xFFFFFFFFull - (key & 0xFFFFFFFFull);
            unsigned int wb = (unsigned int)(key >> 32);
            float wmax;
            std::memcpy(&wmax, &wb, 4);
            const long iot = (long)(idx % nOT), t = (long)((idx / nOT) % T);
            const long ior = (long)((idx / ((unsigned long long)nOT * T)) % nOR);
            const long r = (long)(idx / ((unsigned long long)nOT * T * nOR));
            const long ic = r / (b->ND * b->NP), id = (r / b->NP) % b->ND, is = r % b->NP;
            b->grid.fine_orientation(id, is, ior, o.rot, o.tilt, o.psi);
            o.xoff = pd[0] + b->otx_h[t * nOT + iot];
            o.yoff = pd[1] + b->oty_h[t * nOT + iot];
            o.cls = (double)ic + 1;
            o.pmax = (double)wmax / ps.sum_fine;
            o.best_ihidden_over = ((r * T + t) * nOR + ior) * nOT + iot;
            o.dLL = std::log(ps.sum_fine) - o.fine_min_diff2 - b->logsigma2;
            // four partial sums: no serial dependency chain through wnorm
            double wn[4] = {0., 0., 0., 0.};
            const double *__restrict__ sp = &shell[(size_t)p * nsh];
            const double *__restrict__ pw = &power_h[(size_t)p * nsh];
            for (int i = 0; i < nsh; ++i) {
                wsig[i] += sp[i];
                wn[i & 3] += sp[i];
            }
            for (int i = b->cur / 2 + 1; i < nsh; ++i) {
                wsig[i] += pw[i];
                wn[i & 3] += pw[i];
            }
            const double wnorm = (wn[0] + wn[1]) + (wn[2] + wn[3]);
            o.norm = pd[5];
            if (d.do_norm_correction) {
                o.norm = pd[5] / d.avg_norm_correction * std::sqrt(wnorm * 2.);
                acc.avg_norm += o.norm;
            }
            if (d.do_scale_correction) {
                acc.XA += pacc[(size_t)p * 8 + 2] / pd[6];
                acc.AA += pacc[(size_t)p * 8 + 3] / (pd[6] * pd[6]);
            }
            acc.sumw += pacc[(size_t)p * 8 + 0];
            acc.off += pacc[(size_t)p * 8 + 1];
            acc.LL += o.dLL;
            acc.pmax += o.pmax;
        }
    }
    for (int th = 0; th < nth; ++th)
        if (rs[th].bad >= 0) return fail(GBR_ERR_NUMERICAL, "zero sum of weights for particle " + std::to_string(rs[th].bad));
    {
        double *__restrict__ wsig = b->w_sigma2.data();
        for (int th = 0; th < nth; ++th) {
            const double *src = sig_part.data() + (size_t)th * nsh;
            for (int i = 0; i < nsh; ++i) wsig[i] += src[i];
            const RangeSums &a = rs[th];
            b->w_avg_norm += a.avg_norm;
            b->w_XA += a.XA;
            b->w_AA += a.AA;
            b->w_sumw_group += a.sumw;
            b->w_sigma2_offset += a.off;
            b->w_LL += a.LL;
            b->w_ave_Pmax += a.pmax;
        }
    }
    w->stage_ms[ST_N + 1] +=
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_final).count();
    return GBR_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

size_t gbr_last_error(char *buf, size_t len) {
    if (buf && len) {
        std::strncpy(buf, g_last_error.c_str(), len - 1);
        buf[len - 1] = 0;
    }
    return g_last_error.size();
}

const char *gbr_version(void) { return "libgbrelion 0.1 (sm_103a)"; }

int gbr_bundle_create(const gbr_model_desc *desc, int device, gbr_bundle **out) {
    if (!desc || !out) return fail(GBR_ERR_INVALID, "null argument");
    const gbr_model_desc &d = *desc;
    if (d.ori_size <= 0 || d.nr_classes <= 0 || d.current_size <= 0 || d.coarse_size <= 0 ||
        d.coarse_size > d.current_size || d.current_size > d.ori_size || d.current_size % 2 ||
        d.coarse_size % 2 || d.padding_factor <= 0 || d.pixel_size <= 0 || d.offset_step <= 0 ||
        d.offset_range < 0 || d.sigma2_len <= 0 || d.healpix_order < 0 || d.healpix_order > 8)
        return fail(GBR_ERR_INVALID, "invalid model description");
    if (d.adaptive_oversampling != 1)
        return fail(GBR_ERR_UNSUPPORTED, "only --oversampling 1 is implemented");
    if (d.maximum_significants > 0)
        return fail(GBR_ERR_UNSUPPORTED, "--maxsig is not implemented");
    if (d.precision != GBR_PREC_FP32 && d.precision != GBR_PREC_BF16)
        return fail(GBR_ERR_INVALID, "unknown precision");
    if (d.ref_dim != 0 && d.ref_dim != 2 && d.ref_dim != 3)
        return fail(GBR_ERR_INVALID, "ref_dim must be 2 or 3");
    const bool is2d = d.ref_dim == 2;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
        return fail(GBR_ERR_CUDA, "no CUDA device " + std::to_string(device));
    GBR_CUDA(cudaSetDevice(device));
    std::unique_ptr<gbr_bundle> b(new gbr_bundle());
    b->d = d;
    b->device = device;
    b->is2d = is2d;
    b->grid.build((int)d.healpix_order, d.psi_step, d.offset_range, d.offset_step, (int)d.adaptive_oversampling,
                  !is2d);
    b->K = d.nr_classes;
    b->KP = is2d ? (int)b->K : 1;
    b->ND = b->grid.ndir();
    b->NP = b->grid.npsi();
    b->T = b->grid.ntrans();
    b->R = b->K * b->ND * b->NP;
    b->nOR = b->grid.nover_rot();
    b->nOT = b->grid.nover_trans();
    b->RF = b->R * b->nOR;
    b->TF = b->T * b->nOT;
    if (b->R > 0x7fffffffL / 8) return fail(GBR_ERR_INVALID, "sampling too large");
    b->nshell = (int)(d.ori_size / 2 + 1);
    b->cur = (int)d.current_size;
    b->crs = (int)d.coarse_size;
    b->full_npix = b->cur * (b->cur / 2 + 1);
    b->vol.resize(b->K);
    b->have_vol.assign(b->K, 0);
    // backprojector volumes (BackProjector::initZeros(current_size))
    const int r_max = (int)std::min<int64_t>(d.current_size / 2, d.ori_size / 2);
    const int pad_size = 2 * (iround((double)d.padding_factor * r_max) + 1) + 1;
    // 2D: one padded plane (BackProjector::initialiseDataAndWeight with ref_dim 2)
    b->bg = is2d ? VolGeom{pad_size / 2 + 1, pad_size, 1, -(pad_size / 2), 0, r_max, (int)d.padding_factor, 2}
                 : VolGeom{pad_size / 2 + 1, pad_size, pad_size, -(pad_size / 2), -(pad_size / 2), r_max,
                           (int)d.padding_factor, 3};
    b->bp_vox = (size_t)b->bg.xdim * b->bg.ydim * b->bg.zdim;
    b->bp_data.resize(b->K);
    b->bp_weight.resize(b->K);
    b->bp_stage.resize(b->K);
    std::vector<float4 *> sp(b->K);
    for (long k = 0; k < b->K; ++k) {
        GBR_CUDA(b->bp_data[k].reserve(b->bp_vox));
        GBR_CUDA(b->bp_weight[k].reserve(b->bp_vox));
        GBR_CUDA(b->bp_stage[k].reserve(b->bp_vox));
        GBR_CUDA(b->bp_data[k].zero());
        GBR_CUDA(b->bp_weight[k].zero());
        GBR_CUDA(b->bp_stage[k].zero());
        sp[k] = b->bp_stage[k].p;
    }
    GBR_CUDA(b->bps_ptrs.upload(sp.data(), sp.size()));
    GBR_CUDA(b->w_pdf_cls.reserve(b->K));
    GBR_CUDA(b->w_pdf_dir.reserve((size_t)b->K * b->ND));
    GBR_CUDA(b->w_pdf_cls.zero());
    GBR_CUDA(b->w_pdf_dir.zero());
    if (is2d) {
        b->class_prior_h.assign(2 * b->K, 0.);
        GBR_CUDA(b->class_prior.upload(b->class_prior_h.data(), b->class_prior_h.size()));
        GBR_CUDA(b->w_prior_off.reserve(2 * b->K));
        GBR_CUDA(b->w_prior_off.zero());
    }
    b->w_sigma2.assign(b->nshell, 0.);
    GBR_CUDA(cudaDeviceSynchronize());
    *out = b.release();
    return GBR_OK;
}

int gbr_projector_upload(gbr_bundle *b, int64_t iclass, const float *data, int64_t xdim, int64_t ydim,
                         int64_t zdim, int64_t yinit, int64_t zinit, int64_t r_max, int64_t padding_factor) {
    if (!b || !data || iclass < 0 || iclass >= b->K) return fail(GBR_ERR_INVALID, "bad class or data");
    GBR_LOCK(b);
    ++g_api_gen;
    if (xdim <= 1 || ydim <= 1 || padding_factor != b->d.padding_factor ||
        (b->is2d ? (zdim != 1 || zinit != 0) : zdim <= 1))
        return fail(GBR_ERR_INVALID, "bad projector dimensions");
    if (-yinit + 1 > ydim || -zinit + 1 > zdim || r_max * padding_factor + 1 >= xdim)
        return fail(GBR_ERR_INVALID, "projector origin / r_max outside the volume");
    VolGeom g{(int)xdim, (int)ydim, (int)zdim, (int)yinit, (int)zinit, (int)r_max, (int)padding_factor,
              b->is2d ? 2 : 3};
    bool any = false;
    for (long k = 0; k < b->K; ++k) any |= (k != iclass && b->have_vol[k] != 0);
    if (any && std::memcmp(&g, &b->pg, sizeof(g)) != 0)
        return fail(GBR_ERR_INVALID, "all classes must share one projector geometry");
    GBR_CUDA(cudaSetDevice(b->device));
    b->pg = g;
    GBR_CUDA(b->vol[iclass].upload(reinterpret_cast<const float2 *>(data), (size_t)xdim * ydim * zdim));
    b->have_vol[iclass] = 1;
    b->tables_ready = false;
    return GBR_OK;
}

int gbr_model_set_arrays(gbr_bundle *b, const double *sigma2_noise, const double *pdf_class,
                         const double *pdf_direction, const double *data_vs_prior) {
    if (!b || !sigma2_noise || !pdf_class || !pdf_direction) return fail(GBR_ERR_INVALID, "null array");
    GBR_LOCK(b);
    ++g_api_gen;
    if (b->d.do_scale_correction && !data_vs_prior)
        return fail(GBR_ERR_INVALID, "data_vs_prior needed with scale correction");
    b->sigma2.assign(sigma2_noise, sigma2_noise + b->d.sigma2_len);
    b->pdf_class.assign(pdf_class, pdf_class + b->K);
    b->pdf_dir.assign(pdf_direction, pdf_direction + b->K * b->ND);
    if (data_vs_prior) b->dvp.assign(data_vs_prior, data_vs_prior + b->K * b->nshell);
    b->have_arrays = true;
    b->tables_ready = false;
    return GBR_OK;
}

int gbr_bundle_reserve(gbr_bundle *b, size_t bytes) {
    if (!b) return fail(GBR_ERR_INVALID, "null bundle");
    GBR_LOCK(b);
    ++g_api_gen;
    b->budget = bytes;
    return GBR_OK;
}

int gbr_worker_create(gbr_bundle *b, gbr_worker **out) {
    if (!b || !out) return fail(GBR_ERR_INVALID, "null argument");
    GBR_CUDA(cudaSetDevice(b->device));
    std::unique_ptr<gbr_worker> w(new gbr_worker());
    w->b = b;
    GBR_CUDA(cudaStreamCreateWithFlags(&w->st, cudaStreamNonBlocking));
    for (int i = 0; i <= ST_N; ++i) GBR_CUDA(cudaEventCreate(&w->ev[i]));
    GBR_CUDA(cudaEventCreate(&w->ev_in));
    for (auto &ev : w->ev_img) GBR_CUDA(cudaEventCreate(&ev));
    GBR_CUDA(cudaStreamCreateWithFlags(&w->st_copy, cudaStreamNonBlocking));
    for (auto &sl : w->stage) {
        GBR_CUDA(cudaEventCreate(&sl.start));
        GBR_CUDA(cudaEventCreate(&sl.ready));
        GBR_CUDA(cudaEventCreateWithFlags(&sl.consumed, cudaEventDisableTiming));
    }
    GBR_CUDA(cudaEventCreate(&w->ev_call));
    GBR_CUDA(cudaEventCreateWithFlags(&w->ev_inputs, cudaEventDisableTiming));
    *out = w.release();
    return GBR_OK;
}

int gbr_worker_set_debug(gbr_worker *w, int on) {
    if (!w) return fail(GBR_ERR_INVALID, "null worker");
    ++g_api_gen;
    w->debug = on ? 1 : 0;
    return GBR_OK;
}

int gbr_worker_set_option(gbr_worker *w, int option, int64_t value) {
    if (!w) return fail(GBR_ERR_INVALID, "null worker");
    ++g_api_gen;
    if (value < 0 || value > (1LL << 30)) return fail(GBR_ERR_INVALID, "option value out of range");
    switch (option) {
        case GBR_OPT_DEBUG: w->debug = value ? 1 : 0; break;
        case GBR_OPT_FINE_MODE:
            if (value > 2) return fail(GBR_ERR_INVALID, "fine mode must be 0 (auto), 1 (dense) or 2 (sparse)");
            w->fine_mode = (int)value;
            break;
        case GBR_OPT_COARSE_ROWS:
            if (value > 1) return fail(GBR_ERR_INVALID, "coarse rows must be 0 (skip far rows) or 1 (all)");
            w->coarse_rows = (int)value;
            break;
        case GBR_OPT_CAND_CAP: w->cand_cap_max = value > 0 ? (int)value : (1 << 16); break;
        case GBR_OPT_CAND_BUF: w->cand_buf = (int)value; break;
        case GBR_OPT_BATCH_CAP: w->batch_cap = (int)value; break;
        case GBR_OPT_TILE_GROUP: w->tc_tune.group_m = (int)value; break;
        case GBR_OPT_KEEP_A:
            if (value > 1) return fail(GBR_ERR_INVALID, "keep_a must be 0 or 1");
            w->tc_tune.keep_a = (int)value;
            break;
        case GBR_OPT_PAIR:
            if (value > 1) return fail(GBR_ERR_INVALID, "pair must be 0 or 1");
            w->tc_tune.pair = (int)value;
            break;
        case GBR_OPT_BP_FLUSH: w->bp_flush = (int)value; break;
        case GBR_OPT_BP_DIRECT:
            if (value > 1) return fail(GBR_ERR_INVALID, "bp_direct must be 0 or 1");
            w->bp_direct = (int)value;
            break;
        case GBR_OPT_GRAPH:
            if (value > 1) return fail(GBR_ERR_INVALID, "graph must be 0 or 1");
            w->use_graph = (int)value;
            break;
        default: return fail(GBR_ERR_INVALID, "unknown worker option " + std::to_string(option));
    }
    return GBR_OK;
}

int gbr_expect_batch(gbr_worker *w, const gbr_particle_batch *batch, gbr_particle_result *res) {
    if (!w || !batch || !res || batch->n < 0) return fail(GBR_ERR_INVALID, "null argument");
    GBR_LOCK(w->b);
    if (batch->n == 0) return GBR_OK;
    if (!batch->fimg || !batch->fimg_nomask || !batch->fctf || !batch->power_img || !batch->old_offset ||
        !batch->prior || !batch->highres_Xi2 || !batch->norm_correction || !batch->scale)
        return fail(GBR_ERR_INVALID, "null particle array");
    gbr_bundle *b = w->b;
    GBR_CUDA(cudaSetDevice(b->device));
    const int n_all = (int)batch->n;
    int s = call_capacity(w, n_all);
    if (s) return s;
    const size_t full = (size_t)b->full_npix;
    const cudaMemcpyKind kind = batch->device_resident ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    for (int p0 = 0; p0 < n_all; p0 += w->pass_cap) {
        const int n = std::min(w->pass_cap, n_all - p0);
        GBR_CUDA(cudaEventRecord(w->ev_in, w->st));
        // inputs already in the worker's buffers (gbr_expect_images prepares
        // into them) are not copied
        const float *xs = batch->fimg + 2 * full * p0, *xns = batch->fimg_nomask + 2 * full * p0;
        const float *cs = batch->fctf + full * p0;
        if ((const void *)xs != (const void *)w->X.p)
            GBR_CUDA(cudaMemcpyAsync(w->X.p, xs, sizeof(float2) * full * n, kind, w->st));
        if ((const void *)xns != (const void *)w->Xn.p)
            GBR_CUDA(cudaMemcpyAsync(w->Xn.p, xns, sizeof(float2) * full * n, kind, w->st));
        if ((const void *)cs != (const void *)w->C.p)
            GBR_CUDA(cudaMemcpyAsync(w->C.p, cs, sizeof(float) * full * n, kind, w->st));
        GBR_CUDA(w->h_pdat.reserve((size_t)n * 8));
        GBR_CUDA(w->h_power.reserve((size_t)n * b->nshell));
        double *pdat = w->h_pdat.p, *power = w->h_power.p;
        if (batch->device_resident) {
            // metadata rows gathered on the device; the host copies (for the
            // per-particle finalisation) arrive before the batch's last sync
            GBR_CUDA(launch_gather_pdat(batch->old_offset + 2 * p0, batch->prior + 2 * p0, batch->highres_Xi2 + p0,
                                        batch->norm_correction + p0, batch->scale + p0, n, w->pdat.p, w->st));
            w->launches += 1;
            GBR_CUDA(cudaMemcpyAsync(pdat, w->pdat.p, sizeof(double) * n * 8, cudaMemcpyDeviceToHost, w->st));
            GBR_CUDA(cudaMemcpyAsync(power, batch->power_img + (size_t)b->nshell * p0, sizeof(double) * b->nshell * n,
                                     cudaMemcpyDeviceToHost, w->st));
        } else {
            for (int p = 0; p < n; ++p) {
                const int q = p0 + p;
                pdat[p * 8 + 0] = batch->old_offset[2 * q];
                pdat[p * 8 + 1] = batch->old_offset[2 * q + 1];
                pdat[p * 8 + 2] = batch->prior[2 * q];
                pdat[p * 8 + 3] = batch->prior[2 * q + 1];
                pdat[p * 8 + 4] = batch->highres_Xi2[q];
                pdat[p * 8 + 5] = batch->norm_correction[q];
                pdat[p * 8 + 6] = batch->scale[q];
                pdat[p * 8 + 7] = 0.;
            }
            std::memcpy(power, batch->power_img + (size_t)b->nshell * p0, sizeof(double) * b->nshell * n);
            GBR_CUDA(cudaMemcpyAsync(w->pdat.p, pdat, sizeof(double) * n * 8, cudaMemcpyHostToDevice, w->st));
        }
        w->pass_p0 = p0;
        s = run_batch(w, n, power, pdat, res + p0);
        if (s) return s;
    }
    return GBR_OK;
}

int gbr_orientation_blocks(const gbr_bundle *b, int64_t *nblocks, int64_t *dirs_per_block, int64_t *rows_per_block) {
    if (!b) return fail(GBR_ERR_INVALID, "null bundle");
    int s = restricted_supported(b);
    if (s) return s;
    if (nblocks) *nblocks = b->R / (kDirsPerBlock * b->NP);
    if (dirs_per_block) *dirs_per_block = kDirsPerBlock;
    if (rows_per_block) *rows_per_block = kDirsPerBlock * b->NP;
    return GBR_OK;
}

int gbr_expect_batch_blocks(gbr_worker *w, const gbr_particle_batch *batch, const int32_t *blocks, int64_t m,
                            gbr_particle_result *res) {
    if (!w || !batch || !blocks || m <= 0) return fail(GBR_ERR_INVALID, "null argument or empty block lists");
    GBR_LOCK(w->b);
    int s = restricted_supported(w->b);
    if (s) return s;
    w->restrict_blocks = blocks;
    w->restrict_m = m;
    s = gbr_expect_batch(w, batch, res);
    w->restrict_blocks = nullptr;
    w->restrict_m = 0;
    return s;
}

int gbr_bundle_set_optics(gbr_bundle *b, const gbr_optics_desc *optics) {
    if (!b || !optics) return fail(GBR_ERR_INVALID, "null argument");
    GBR_LOCK(b);
    ++g_api_gen;
    if (!(optics->kV > 0.) || optics->Q0 < 0. || optics->Q0 >= 1. || !(optics->particle_diameter > 0.) ||
        !(optics->width_mask_edge > 0.))
        return fail(GBR_ERR_INVALID, "invalid optics / mask parameters");
    b->optics = *optics;
    b->have_optics = true;
    return GBR_OK;
}

namespace {

// getFourierTransformsAndCtfs for a whole batch into the given device arrays.
int prepare_images(gbr_worker *w, const gbr_image_batch *in, float2 *fimg, float2 *fnm, float *fctf, double *power,
                   double *xi2, double *off_out, const float *staged_images = nullptr) {
    gbr_bundle *b = w->b;
    if (!b->have_optics) return fail(GBR_ERR_STATE, "optics not set (gbr_bundle_set_optics)");
    const int n = (int)in->n, N = (int)b->d.ori_size, cur = b->cur;
    if (n <= 0) return GBR_OK;
    if (n > 4096) return fail(GBR_ERR_INVALID, "gbr_prepare_images: at most 4096 images per call");
    if (!in->images || !in->old_offset || !in->norm_correction || !in->ctf)
        return fail(GBR_ERR_INVALID, "null image batch array");
    cudaStream_t st = w->st;
    const size_t npx = (size_t)n * N * N, nf = (size_t)n * N * (N / 2 + 1);
    GBR_CUDA(w->pi_A.reserve(npx));
    GBR_CUDA(w->pi_B.reserve(npx));
    GBR_CUDA(w->pi_FA.reserve(nf));
    GBR_CUDA(w->pi_FB.reserve(nf));
    GBR_CUDA(w->pi_bg.reserve((size_t)2 * n));
    GBR_CUDA(w->pi_W.reserve((size_t)N * N));
    GBR_CUDA(w->pi_ctf.reserve((size_t)n * 6));
    GBR_CUDA(w->pi_shift.reserve((size_t)n * 2));
    GBR_CUDA(w->pi_factor.reserve(n));
    // rounded old offsets (selfROUND, src/ml_optimiser.cpp:6054) and norm factors on the host
    std::vector<double> off((size_t)n * 2), nc(n);
    if (in->device_resident) {
        GBR_CUDA(cudaMemcpy(off.data(), in->old_offset, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost));
        GBR_CUDA(cudaMemcpy(nc.data(), in->norm_correction, sizeof(double) * n, cudaMemcpyDeviceToHost));
    } else {
        std::memcpy(off.data(), in->old_offset, sizeof(double) * 2 * n);
        std::memcpy(nc.data(), in->norm_correction, sizeof(double) * n);
    }
    std::vector<int> sh((size_t)n * 2);
    std::vector<float> fac(n);
    std::vector<double> offr((size_t)n * 2);
    for (int p = 0; p < n; ++p) {
        for (int k = 0; k < 2; ++k) {
            const double v = off[2 * p + k];
            sh[2 * p + k] = v > 0 ? (int)(v + 0.5) : (int)(v - 0.5);
            offr[2 * p + k] = sh[2 * p + k];
        }
        fac[p] = b->d.do_norm_correction ? (float)(b->d.avg_norm_correction / nc[p]) : 1.f;
    }
    GBR_CUDA(cudaMemcpyAsync(w->pi_shift.p, sh.data(), sizeof(int) * sh.size(), cudaMemcpyHostToDevice, st));
    GBR_CUDA(cudaMemcpyAsync(w->pi_factor.p, fac.data(), sizeof(float) * n, cudaMemcpyHostToDevice, st));
    GBR_CUDA(cudaMemcpyAsync(off_out, offr.data(), sizeof(double) * offr.size(), cudaMemcpyHostToDevice, st));
    GBR_CUDA(cudaMemcpyAsync(w->pi_ctf.p, in->ctf, sizeof(double) * 6 * n,
                             in->device_resident ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
    const float *imgs = staged_images ? staged_images : in->images;
    GBR_CUDA(cudaEventRecord(w->ev_img[0], st));
    if (!in->device_resident && !staged_images) {
        GBR_CUDA(w->pi_images.reserve(npx));
        GBR_CUDA(cudaMemcpyAsync(w->pi_images.p, in->images, sizeof(float) * npx, cudaMemcpyHostToDevice, st));
        imgs = w->pi_images.p;
    }
    GBR_CUDA(cudaEventRecord(w->ev_img[1], st));
    if (w->fft_plan < 0 || w->fft_N != N || w->fft_batch != n) {
        if (w->fft_plan >= 0) destroy_fft_plan(w->fft_plan);
        w->fft_plan = -1;
        if (make_fft_plan(N, n, &w->fft_plan)) return fail(GBR_ERR_CUDA, "cuFFT plan creation failed");
        w->fft_N = N;
        w->fft_batch = n;
    }
    PrepImagesArgs a{};
    a.n = n;
    a.N = N;
    a.cur = cur;
    a.images = imgs;
    a.shift = w->pi_shift.p;
    a.factor = w->pi_factor.p;
    a.ctf = w->pi_ctf.p;
    a.pixel = b->d.pixel_size;
    a.kV = b->optics.kV;
    a.Cs = b->optics.Cs;
    a.Q0 = b->optics.Q0;
    a.mask_radius = b->optics.particle_diameter / (2. * b->d.pixel_size);
    a.mask_width = b->optics.width_mask_edge;
    a.A = w->pi_A.p;
    a.B = w->pi_B.p;
    a.FA = w->pi_FA.p;
    a.FB = w->pi_FB.p;
    a.bg = w->pi_bg.p;
    a.W = w->pi_W.p;
    a.mask_fresh = (w->pi_W_key[0] != N || w->pi_W_key[1] != a.mask_radius || w->pi_W_key[2] != a.mask_width) ? 1 : 0;
    w->pi_W_key[0] = N;
    w->pi_W_key[1] = a.mask_radius;
    w->pi_W_key[2] = a.mask_width;
    a.fft_plan = w->fft_plan;
    a.fimg = fimg;
    a.fimg_nomask = fnm;
    a.fctf = fctf;
    a.power = power;
    a.xi2 = xi2;
    GBR_CUDA(launch_prepare_images(a, st));
    GBR_CUDA(cudaEventRecord(w->ev_img[2], st));
    w->launches += 6 + a.mask_fresh;  // own kernels (the cuFFT launches are the library's)
    return GBR_OK;
}

}  // namespace

int gbr_prepare_images(gbr_worker *w, const gbr_image_batch *in, void *fimg, void *fimg_nomask, float *fctf,
                       double *power_img, double *highres_Xi2, double *old_offset_rounded) {
    if (!w || !in || !fimg || !fimg_nomask || !fctf || !power_img || !highres_Xi2 || !old_offset_rounded)
        return fail(GBR_ERR_INVALID, "null argument");
    GBR_LOCK(w->b);
    GBR_CUDA(cudaSetDevice(w->b->device));
    int s = prepare_images(w, in, static_cast<float2 *>(fimg), static_cast<float2 *>(fimg_nomask), fctf, power_img,
                           highres_Xi2, old_offset_rounded);
    if (s) return s;
    GBR_CUDA(cudaStreamSynchronize(w->st));
    return GBR_OK;
}

namespace {

// Issue a requested staging copy on the copy stream, after the previous
// batch in the slot has been read.
int issue_stage(gbr_worker *w, gbr_worker::StageSlot &sl, cudaEvent_t after = nullptr) {
    if (sl.used) GBR_CUDA(cudaStreamWaitEvent(w->st_copy, sl.consumed, 0));
    if (after) GBR_CUDA(cudaStreamWaitEvent(w->st_copy, after, 0));
    GBR_CUDA(cudaEventRecord(sl.start, w->st_copy));
    GBR_CUDA(cudaMemcpyAsync(sl.img.p, sl.host, sizeof(float) * sl.npx, cudaMemcpyHostToDevice, w->st_copy));
    GBR_CUDA(cudaEventRecord(sl.ready, w->st_copy));
    sl.pending = false;
    return GBR_OK;
}

// Issue every requested staging copy, oldest first, to start once the event
// `after` (recorded on the compute stream behind the current call's host-to-
// device copies) has completed.  The device's host-to-device copies run one
// after the other across streams: a batch copy issued ahead of the call's
// small input copies held them, and the E-step behind them, for the whole
// upload (measured).
int pump_stages(gbr_worker *w, cudaEvent_t after) {
    gbr_worker::StageSlot *a = &w->stage[0], *b = &w->stage[1];
    if (b->seq < a->seq) std::swap(a, b);
    for (gbr_worker::StageSlot *sl : {a, b})
        if (sl->pending) {
            int s = issue_stage(w, *sl, after);
            if (s) return s;
        }
    return GBR_OK;
}

}  // namespace

int gbr_stage_images(gbr_worker *w, const gbr_image_batch *in) {
    if (!w || !in || !in->images) return fail(GBR_ERR_INVALID, "null argument");
    GBR_LOCK(w->b);
    if (in->device_resident) return fail(GBR_ERR_INVALID, "gbr_stage_images: host batches only");
    gbr_bundle *b = w->b;
    GBR_CUDA(cudaSetDevice(b->device));
    const int N = (int)b->d.ori_size;
    if (in->n <= 0 || in->n > 4096) return fail(GBR_ERR_INVALID, "gbr_stage_images: 1 to 4096 images");
    gbr_worker::StageSlot &sl = w->stage[w->stage_next];
    w->stage_next ^= 1;
    const size_t npx = (size_t)in->n * N * N;
    if (sl.img.n < npx) {
        // a larger slot: the previous copy into it and its readers must be done
        GBR_CUDA(cudaStreamSynchronize(w->st_copy));
        GBR_CUDA(cudaStreamSynchronize(w->st));
        GBR_CUDA(sl.img.reserve(npx));
    }
    // the copy itself is issued by the next gbr_expect_images once that call's
    // own input copies are queued (or at once if it asks for this batch)
    sl.host = in->images;
    sl.n = in->n;
    sl.npx = npx;
    sl.seq = ++w->stage_seq;
    sl.valid = true;
    sl.pending = true;
    return GBR_OK;
}

int gbr_expect_images(gbr_worker *w, const gbr_image_batch *in, gbr_particle_result *res) {
    if (!w || !in || !res) return fail(GBR_ERR_INVALID, "null argument");
    GBR_LOCK(w->b);
    if (in->n == 0) return GBR_OK;
    if (!in->prior || !in->scale) return fail(GBR_ERR_INVALID, "null image batch array");
    gbr_bundle *b = w->b;
    GBR_CUDA(cudaSetDevice(b->device));
    const size_t n = (size_t)in->n, cur = (size_t)b->cur, X = cur / 2 + 1, half = (size_t)b->nshell;
    int s = call_capacity(w, (int)n);
    if (s) return s;
    // a call that fits one pass prepares straight into the E-step's input
    // buffers (no device-to-device copies of the Fourier images)
    const bool in_place = (size_t)w->pass_cap >= n;
    if (!in_place) {
        GBR_CUDA(w->pi_fimg.reserve(n * cur * X));
        GBR_CUDA(w->pi_fnm.reserve(n * cur * X));
        GBR_CUDA(w->pi_fctf.reserve(n * cur * X));
    }
    float2 *fimg = in_place ? w->X.p : w->pi_fimg.p, *fnm = in_place ? w->Xn.p : w->pi_fnm.p;
    float *fctf = in_place ? w->C.p : w->pi_fctf.p;
    GBR_CUDA(w->pi_power.reserve(n * half));
    GBR_CUDA(w->pi_xi2.reserve(n));
    GBR_CUDA(w->pi_off.reserve(2 * n));
    GBR_CUDA(w->pi_prior.reserve(2 * n));
    GBR_CUDA(w->pi_norm.reserve(n));
    GBR_CUDA(w->pi_scale.reserve(n));
    gbr_worker::StageSlot *slot = nullptr;
    for (auto &sl : w->stage)
        if (sl.valid && !in->device_resident && sl.host == in->images && sl.n == in->n &&
            (!slot || sl.seq < slot->seq))
            slot = &sl;
    if (slot) {
        if (slot->pending) {
            int s = issue_stage(w, *slot);
            if (s) return s;
        }
        GBR_CUDA(cudaEventRecord(w->ev_call, w->st));
        GBR_CUDA(cudaStreamWaitEvent(w->st, slot->ready, 0));
    }
    s = prepare_images(w, in, fimg, fnm, fctf, w->pi_power.p, w->pi_xi2.p, w->pi_off.p, slot ? slot->img.p : nullptr);
    if (s) return s;
    if (slot) {
        // the preparation kernels have read the slot: it may be refilled
        GBR_CUDA(cudaEventRecord(slot->consumed, w->st));
        slot->valid = false;
        slot->used = true;
    }
    GBR_CUDA(cudaEventSynchronize(w->ev_img[2]));
    float t0 = 0.f, t1 = 0.f;
    cudaEventElapsedTime(&t0, w->ev_img[0], w->ev_img[1]);
    cudaEventElapsedTime(&t1, w->ev_img[1], w->ev_img[2]);
    w->stage_ms[ST_N + 2] += t0;
    w->stage_ms[ST_N + 3] += t1;
    if (slot) {
        // the preparation waited for the slot: both intervals have ended
        float tc = 0.f, tw = 0.f;
        cudaEventElapsedTime(&tc, slot->start, slot->ready);
        cudaEventElapsedTime(&tw, w->ev_call, w->ev_img[0]);
        w->stage_ms[ST_N + 4] += tc;
        w->stage_ms[ST_N + 5] += tw;
    }
    const cudaMemcpyKind kind = in->device_resident ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    GBR_CUDA(cudaMemcpyAsync(w->pi_prior.p, in->prior, sizeof(double) * 2 * n, kind, w->st));
    GBR_CUDA(cudaMemcpyAsync(w->pi_norm.p, in->norm_correction, sizeof(double) * n, kind, w->st));
    GBR_CUDA(cudaMemcpyAsync(w->pi_scale.p, in->scale, sizeof(double) * n, kind, w->st));
    // batches staged for the next calls upload during this call's E-step,
    // behind the call's own host-to-device copies
    GBR_CUDA(cudaEventRecord(w->ev_inputs, w->st));
    s = pump_stages(w, w->ev_inputs);
    if (s) return s;
    gbr_particle_batch pb{};
    pb.n = in->n;
    pb.device_resident = 1;
    pb.fimg = reinterpret_cast<const float *>(fimg);
    pb.fimg_nomask = reinterpret_cast<const float *>(fnm);
    pb.fctf = fctf;
    pb.power_img = w->pi_power.p;
    pb.old_offset = w->pi_off.p;
    pb.prior = w->pi_prior.p;
    pb.highres_Xi2 = w->pi_xi2.p;
    pb.norm_correction = w->pi_norm.p;
    pb.scale = w->pi_scale.p;
    return gbr_expect_batch(w, &pb, res);
}

int gbr_sampling_sizes(const gbr_bundle *b, int64_t *ndir, int64_t *npsi, int64_t *ntrans, int64_t *nover_rot,
                       int64_t *nover_trans) {
    if (!b) return fail(GBR_ERR_INVALID, "null bundle");
    if (ndir) *ndir = b->ND;
    if (npsi) *npsi = b->NP;
    if (ntrans) *ntrans = b->T;
    if (nover_rot) *nover_rot = b->nOR;
    if (nover_trans) *nover_trans = b->nOT;
    return GBR_OK;
}

int64_t gbr_worker_debug_fetch(gbr_worker *w, int what, int64_t i, void *host, int64_t capacity) {
    if (!w || !host) return fail(GBR_ERR_INVALID, "null argument");
    if (!w->debug) return fail(GBR_ERR_STATE, "debug read-back needs gbr_worker_set_debug before the call");
    if (i < 0 || i >= w->dbg_n) return fail(GBR_ERR_INVALID, "particle index out of range");
    // the pass that held particle i of the call
    size_t ip = 0;
    while (i >= w->dbg[ip].n) i -= w->dbg[ip++].n;
    const gbr_worker::DbgPass &D = w->dbg[ip];
    gbr_bundle *b = w->b;
    const long long RT = (long long)b->R * b->T;
    const int nOR = (int)b->nOR, nOT = (int)b->nOT, T = (int)b->T;
    if (what == 0 || what == 1) {
        if (capacity < RT) return fail(GBR_ERR_INVALID, "capacity too small");
        double *o = static_cast<double *>(host);
        const float *src = (what == 0 ? D.coarse.data() : D.wcoarse.data()) + (size_t)i * RT;
        if (what == 1) {
            for (long long e = 0; e < RT; ++e) o[e] = (double)src[e];
            return RT;
        }
        // sparse stores: the segments (32 consecutive columns of the pass's
        // [particle][translation] axis) the coarse pass did not store are
        // reported as +inf (poses beyond the skip distance)
        const long long c0 = ((long long)i * T) >> 5;
        for (long long e = 0; e < RT; ++e) {
            const long long r = e / T, t = e % T;
            bool stored = true;
            if (D.sparse) {
                const unsigned int seg = D.segmask[(size_t)i * b->R + r];
                stored = (seg >> ((((long long)i * T + t) >> 5) - c0)) & 1u;
            }
            o[e] = (stored && std::isfinite(src[e])) ? D.cc[i] + (double)src[e] : INFINITY;
        }
        return RT;
    }
    const long long b0 = D.segf[i], b1 = D.segf[i + 1];
    if (capacity < b1 - b0) return fail(GBR_ERR_INVALID, "capacity too small");
    if (D.dense) {
        // dense layout [rf][tf]: report the computed (finite diff2) entries
        const long long TF = (long long)T * nOT;
        long long m = 0;
        for (long long e = b0; e < b1; ++e) {
            if (!std::isfinite(D.fine[e])) continue;
            const long long loc = e - b0, rf = loc / TF, tf = loc % TF;
            const long long r = rf / nOR, ior = rf % nOR, t = tf / nOT, iot = tf % nOT;
            if (what == 2) static_cast<int64_t *>(host)[m] = ((r * T + t) * nOR + ior) * nOT + iot;
            else if (what == 3) static_cast<double *>(host)[m] = D.cf[i] + (double)D.fine[e];
            else if (what == 4) static_cast<double *>(host)[m] = (double)D.wfine[e];
            else return fail(GBR_ERR_INVALID, "unknown debug selector");
            ++m;
        }
        return m;
    }
    for (long long e = b0; e < b1; ++e) {
        const long long k = e - b0;
        if (what == 2) {
            const FineJob &j = D.jobs[D.ejob[e]];
            const unsigned code = D.ecode[e];
            const long long t = code / (nOR * nOT), ior = (code / nOT) % nOR, iot = code % nOT;
            static_cast<int64_t *>(host)[k] = (((long long)j.r * T + t) * nOR + ior) * nOT + iot;
        } else if (what == 3) {
            static_cast<double *>(host)[k] = D.cf[i] + (double)D.fine[e];
        } else if (what == 4) {
            static_cast<double *>(host)[k] = (double)D.wfine[e];
        } else {
            return fail(GBR_ERR_INVALID, "unknown debug selector");
        }
    }
    return b1 - b0;
}

int gbr_backprojector_dims(const gbr_bundle *b, int64_t *xdim, int64_t *ydim, int64_t *zdim, int64_t *yinit,
                           int64_t *zinit, int64_t *r_max) {
    if (!b) return fail(GBR_ERR_INVALID, "null bundle");
    if (xdim) *xdim = b->bg.xdim;
    if (ydim) *ydim = b->bg.ydim;
    if (zdim) *zdim = b->bg.zdim;
    if (yinit) *yinit = b->bg.yinit;
    if (zinit) *zinit = b->bg.zinit;
    if (r_max) *r_max = b->bg.r_max;
    return GBR_OK;
}

int gbr_backprojector_download(gbr_bundle *b, int64_t iclass, double *data, double *weight) {
    if (!b || iclass < 0 || iclass >= b->K) return fail(GBR_ERR_INVALID, "bad class");
    GBR_LOCK(b);
    GBR_CUDA(cudaSetDevice(b->device));
    int s = flush_staged(b);
    if (s) return s;
    if (data) GBR_CUDA(cudaMemcpy(data, b->bp_data[iclass].p, sizeof(double2) * b->bp_vox, cudaMemcpyDeviceToHost));
    if (weight) GBR_CUDA(cudaMemcpy(weight, b->bp_weight[iclass].p, sizeof(double) * b->bp_vox, cudaMemcpyDeviceToHost));
    return GBR_OK;
}

int gbr_backprojector_upload(gbr_bundle *b, int64_t iclass, const double *data, const double *weight) {
    if (!b || !data || !weight || iclass < 0 || iclass >= b->K) return fail(GBR_ERR_INVALID, "bad class or data");
    GBR_LOCK(b);
    GBR_CUDA(cudaSetDevice(b->device));
    int s = flush_staged(b);
    if (s) return s;
    GBR_CUDA(cudaMemcpy(b->bp_data[iclass].p, data, sizeof(double2) * b->bp_vox, cudaMemcpyHostToDevice));
    GBR_CUDA(cudaMemcpy(b->bp_weight[iclass].p, weight, sizeof(double) * b->bp_vox, cudaMemcpyHostToDevice));
    return GBR_OK;
}

namespace {
int recon_begin(gbr_bundle *b, int64_t iclass) {
    if (!b || iclass < 0 || iclass >= b->K) return fail(GBR_ERR_INVALID, "bad class");
    GBR_CUDA(cudaSetDevice(b->device));
    int s = flush_staged(b);
    if (s) return s;
    if (!b->recon) b->recon = gbr::recon_work_create();
    return GBR_OK;
}
}  // namespace

int gbr_recon_set_precision(gbr_bundle *b, int precision) {
    if (!b) return fail(GBR_ERR_INVALID, "null bundle");
    GBR_LOCK(b);
    int st = recon_begin(b, 0);
    if (st) return st;
    if (precision != GBR_RECON_FP64 && precision != GBR_RECON_FP32)
        return fail(GBR_ERR_INVALID, "unknown reconstruction precision");
    gbr::recon_set_fp32(b->recon, precision == GBR_RECON_FP32);
    return GBR_OK;
}

int gbr_backprojector_symmetrise(gbr_bundle *b, int64_t iclass) {
    if (!b) return fail(GBR_ERR_INVALID, "null bundle");
    GBR_LOCK(b);
    int st = recon_begin(b, iclass);
    if (st) return st;
    return gbr::recon_symmetrise(b->bp_data[iclass].p, b->bp_weight[iclass].p, b->bg);
}

int gbr_update_ssnr(gbr_bundle *b, int64_t iclass, double tau2_fudge, double *tau2_io, double *sigma2_out,
                    double *data_vs_prior_out, double *fourier_coverage_out, const double *fsc,
                    int update_tau2_with_fsc, int is_whole_instead_of_half) {
    if (!b) return fail(GBR_ERR_INVALID, "null bundle");
    GBR_LOCK(b);
    int st = recon_begin(b, iclass);
    if (st) return st;
    if (!tau2_io || (update_tau2_with_fsc && !fsc)) return fail(GBR_ERR_INVALID, "null tau2 / fsc");
    return gbr::recon_update_ssnr(b->recon, b->bp_weight[iclass].p, b->bg, (int)b->d.ori_size, tau2_fudge, tau2_io,
                                  sigma2_out, data_vs_prior_out, fourier_coverage_out, fsc, update_tau2_with_fsc,
                                  is_whole_instead_of_half);
}

int gbr_reconstruct(gbr_bundle *b, int64_t iclass, const gbr_recon_params *p, const double *tau2, double *vol_out) {
    if (!b) return fail(GBR_ERR_INVALID, "null bundle");
    GBR_LOCK(b);
    int st = recon_begin(b, iclass);
    if (st) return st;
    if (!p) return fail(GBR_ERR_INVALID, "null argument");
    const gbr::ReconParams rp{p->max_iter_preweight, p->do_map, p->skip_gridding, p->minres_map, p->tau2_fudge,
                              p->normalise};
    return gbr::recon_reconstruct(b->recon, b->bp_data[iclass].p, b->bp_weight[iclass].p, b->bg,
                                  (int)b->d.ori_size, rp, tau2, vol_out);
}

int gbr_projector_from_map(gbr_bundle *b, int64_t iclass, const double *vol, int64_t current_size,
                           int do_gridding, int64_t min_ires, double *power_spectrum) {
    if (!b) return fail(GBR_ERR_INVALID, "null bundle");
    GBR_LOCK(b);
    ++g_api_gen;
    int st = recon_begin(b, iclass);
    if (st) return st;
    const int dim = b->is2d ? 2 : 3;
    const gbr::VolGeom g = gbr::projector_geometry((int)b->d.ori_size, dim, (int)b->d.padding_factor,
                                                   (int)current_size);
    bool any = false;
    for (long k = 0; k < b->K; ++k) any |= (k != iclass && b->have_vol[k] != 0);
    if (any && std::memcmp(&g, &b->pg, sizeof(g)) != 0)
        return fail(GBR_ERR_INVALID, "all classes must share one projector geometry");
    GBR_CUDA(b->vol[iclass].reserve((size_t)g.xdim * g.ydim * g.zdim));
    st = gbr::recon_projector_from_map(b->recon, vol, (int)b->d.ori_size, dim, (int)b->d.padding_factor, g,
                                       do_gridding, (int)min_ires, b->vol[iclass].p, power_spectrum);
    if (st) return st;
    b->pg = g;
    b->have_vol[iclass] = 1;
    b->tables_ready = false;
    return GBR_OK;
}

int gbr_projector_download(gbr_bundle *b, int64_t iclass, float *data, int64_t *dims) {
    if (!b || !dims || iclass < 0 || iclass >= b->K) return fail(GBR_ERR_INVALID, "bad class");
    GBR_LOCK(b);
    if (!b->have_vol[iclass]) return fail(GBR_ERR_STATE, "no projector for this class");
    const gbr::VolGeom &g = b->pg;
    const int64_t v[7] = {g.xdim, g.ydim, g.zdim, g.yinit, g.zinit, g.r_max, g.pad};
    std::copy(v, v + 7, dims);
    if (data) {
        GBR_CUDA(cudaSetDevice(b->device));
        GBR_CUDA(cudaDeviceSynchronize());
        GBR_CUDA(cudaMemcpy(data, b->vol[iclass].p, sizeof(float2) * (size_t)g.xdim * g.ydim * g.zdim,
                            cudaMemcpyDeviceToHost));
    }
    return GBR_OK;
}

int gbr_fsc(gbr_bundle *b, const double *map1, const double *map2, double *fsc) {
    if (!b) return fail(GBR_ERR_INVALID, "null bundle");
    GBR_LOCK(b);
    int st = recon_begin(b, 0);
    if (st) return st;
    if (!map1 || !map2 || !fsc) return fail(GBR_ERR_INVALID, "null argument");
    return gbr::recon_fsc(b->recon, map1, map2, (int)b->d.ori_size, b->is2d ? 2 : 3, fsc);
}

int gbr_wsum_download(gbr_bundle *b, gbr_wsum *out) {
    if (!b || !out) return fail(GBR_ERR_INVALID, "null argument");
    GBR_LOCK(b);
    GBR_CUDA(cudaSetDevice(b->device));
    GBR_CUDA(cudaDeviceSynchronize());
    if (out->sigma2_noise)
        for (int i = 0; i < b->nshell; ++i) out->sigma2_noise[i] += b->w_sigma2[i];
    if (out->pdf_class) {
        std::vector<double> v(b->K);
        GBR_CUDA(cudaMemcpy(v.data(), b->w_pdf_cls.p, sizeof(double) * b->K, cudaMemcpyDeviceToHost));
        for (long k = 0; k < b->K; ++k) out->pdf_class[k] += v[k];
    }
    if (out->pdf_direction) {
        std::vector<double> v((size_t)b->K * b->ND);
        GBR_CUDA(cudaMemcpy(v.data(), b->w_pdf_dir.p, sizeof(double) * v.size(), cudaMemcpyDeviceToHost));
        for (size_t k = 0; k < v.size(); ++k) out->pdf_direction[k] += v[k];
    }
    out->sigma2_offset += b->w_sigma2_offset;
    out->sumw_group += b->w_sumw_group;
    out->LL += b->w_LL;
    out->ave_Pmax += b->w_ave_Pmax;
    out->avg_norm_correction += b->w_avg_norm;
    out->wsum_signal_product += b->w_XA;
    out->wsum_reference_power += b->w_AA;
    return GBR_OK;
}

int gbr_wsum_download_class_offsets(gbr_bundle *b, double *out) {
    if (!b || !out) return fail(GBR_ERR_INVALID, "null argument");
    GBR_LOCK(b);
    if (!b->is2d) return fail(GBR_ERR_STATE, "class offset priors exist only for 2D classification");
    GBR_CUDA(cudaSetDevice(b->device));
    GBR_CUDA(cudaDeviceSynchronize());
    std::vector<double> v(2 * b->K);
    GBR_CUDA(cudaMemcpy(v.data(), b->w_prior_off.p, sizeof(double) * v.size(), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < v.size(); ++i) out[i] += v[i];
    return GBR_OK;
}

int gbr_model_set_class_offsets(gbr_bundle *b, const double *prior_offset_class) {
    if (!b || !prior_offset_class) return fail(GBR_ERR_INVALID, "null argument");
    GBR_LOCK(b);
    ++g_api_gen;
    if (!b->is2d) return fail(GBR_ERR_STATE, "class offset priors exist only for 2D classification");
    GBR_CUDA(cudaSetDevice(b->device));
    b->class_prior_h.assign(prior_offset_class, prior_offset_class + 2 * b->K);
    GBR_CUDA(b->class_prior.upload(b->class_prior_h.data(), b->class_prior_h.size()));
    return GBR_OK;
}

int gbr_bundle_reset_wsum(gbr_bundle *b) {
    if (!b) return fail(GBR_ERR_INVALID, "null bundle");
    GBR_LOCK(b);
    GBR_CUDA(cudaSetDevice(b->device));
    GBR_CUDA(cudaDeviceSynchronize());
    for (long k = 0; k < b->K; ++k) {
        GBR_CUDA(b->bp_data[k].zero());
        GBR_CUDA(b->bp_weight[k].zero());
        if (b->staged) GBR_CUDA(b->bp_stage[k].zero());
    }
    b->staged = 0;
    GBR_CUDA(b->w_pdf_cls.zero());
    GBR_CUDA(b->w_pdf_dir.zero());
    if (b->is2d) GBR_CUDA(b->w_prior_off.zero());
    std::fill(b->w_sigma2.begin(), b->w_sigma2.end(), 0.);
    b->w_sigma2_offset = b->w_sumw_group = b->w_LL = b->w_ave_Pmax = b->w_avg_norm = b->w_XA = b->w_AA = 0.;
    GBR_CUDA(cudaDeviceSynchronize());
    return GBR_OK;
}

int gbr_worker_stage_times(const gbr_worker *w, double *ms, int64_t n, int64_t *n_written) {
    if (!w || !ms) return fail(GBR_ERR_INVALID, "null argument");
    const int64_t m = std::min<int64_t>(n, ST_N + 6);
    for (int64_t i = 0; i < m; ++i) ms[i] = w->stage_ms[i];
    if (n_written) *n_written = m;
    return GBR_OK;
}

int gbr_worker_launch_count(const gbr_worker *w, int64_t *count) {
    if (!w || !count) return fail(GBR_ERR_INVALID, "null argument");
    *count = w->launches;
    return GBR_OK;
}

int gbr_worker_graph_stats(const gbr_worker *w, int64_t *captures, int64_t *replays) {
    if (!w) return fail(GBR_ERR_INVALID, "null worker");
    if (captures) *captures = w->g_captures;
    if (replays) *replays = w->g_replays;
    return GBR_OK;
}

int gbr_measure_fp32_peak(int device, double *tflops) {
    if (!tflops) return fail(GBR_ERR_INVALID, "null argument");
    GBR_CUDA(cudaSetDevice(device));
    float ms = 0.f;
    double flops = 0.;
    GBR_CUDA(gbr::launch_fp32_probe(&ms, &flops));
    *tflops = flops / (ms * 1e-3) / 1e12;
    return GBR_OK;
}

int gbr_worker_destroy(gbr_worker *w) {
    if (!w) return GBR_OK;
    cudaSetDevice(w->b->device);
    if (w->st) cudaStreamSynchronize(w->st);
    for (int i = 0; i <= ST_N; ++i)
        if (w->ev[i]) cudaEventDestroy(w->ev[i]);
    if (w->ev_in) cudaEventDestroy(w->ev_in);
    for (auto &ev : w->ev_img)
        if (ev) cudaEventDestroy(ev);
    if (w->st_copy) cudaStreamSynchronize(w->st_copy);
    if (w->ev_call) cudaEventDestroy(w->ev_call);
    if (w->ev_inputs) cudaEventDestroy(w->ev_inputs);
    for (auto &sl : w->stage) {
        if (sl.start) cudaEventDestroy(sl.start);
        if (sl.ready) cudaEventDestroy(sl.ready);
        if (sl.consumed) cudaEventDestroy(sl.consumed);
    }
    if (w->st_copy) cudaStreamDestroy(w->st_copy);
    if (w->fft_plan >= 0) destroy_fft_plan(w->fft_plan);
    if (w->gexec) cudaGraphExecDestroy(w->gexec);
    if (w->st) cudaStreamDestroy(w->st);
    delete w;
    return GBR_OK;
}

int gbr_bundle_destroy(gbr_bundle *b) {
    if (!b) return GBR_OK;
    cudaSetDevice(b->device);
    cudaDeviceSynchronize();
    for (gbr::VolTexture &t : b->vtex) gbr::vol_texture_release(t);
    delete b;
    return GBR_OK;
}

// ---- learned pose proposal (k_posenet.cu) --------------------------------
struct gbr_posenet {
    gbr_bundle *b = nullptr;
    gbr::PnDims d;  // d.B = batch capacity
    int nbins = 0;
    uint64_t seed = 0;
    long long t = 0;  // Adam steps taken
    cudaStream_t st = nullptr;
    DevBuf<float> params, grad, m, v;
    DevBuf<int> bin;
    DevBuf<float> inv_cnt;
    DevBuf<float> pw, feat, a1, a2, h, logits, dl, d1, d2, loss, target, ctf_pool, prob;
    DevBuf<float> feat_all, target_all;  // training on particle images with given targets
    DevBuf<float> bw_scratch;            // partial weight gradients of the convolutions
    DevBuf<float> mass;                  // proposed blocks' probability per particle
    DevBuf<int> label, idx;
    DevBuf<float2> fimg;
    ~gbr_posenet() {
        if (st) cudaStreamDestroy(st);
    }
};

namespace {

uint64_t host_mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// features of count prepared images (host) into n->feat (device), count <= d.B
int pn_features_dev(gbr_posenet *n, const float *fimg, int count) {
    gbr_bundle *b = n->b;
    const size_t full = (size_t)b->full_npix;
    // host or device images (the copy's direction from the unified address)
    GBR_CUDA(cudaMemcpyAsync(n->fimg.p, fimg, sizeof(float2) * full * count, cudaMemcpyDefault, n->st));
    GBR_CUDA(gbr::pn_power(n->fimg.p, (int)full, b->pc.p, b->nc, b->minv_c.p, count, n->pw.p, n->st));
    GBR_CUDA(gbr::pn_bin(n->pw.p, b->nc, n->bin.p, n->inv_cnt.p, n->nbins, count, n->feat.p, n->st));
    return GBR_OK;
}

}  // namespace

int gbr_posenet_create(gbr_bundle *b, const gbr_posenet_desc *desc, gbr_posenet **out) {
    if (!b || !desc || !out) return fail(GBR_ERR_INVALID, "null argument");
    GBR_CUDA(cudaSetDevice(b->device));
    int s = build_tables(b);
    if (s) return s;
    if (desc->nring < 1 || desc->nring > b->crs / 2 || desc->nangle < 5 || desc->nangle > 256 || desc->c1 < 1 ||
        desc->c1 > 32 || desc->c2 < 1 || desc->c2 > 32 || desc->max_batch < 1 || desc->max_batch > 65536)
        return fail(GBR_ERR_INVALID,
                    "gbr_posenet_create: invalid sizes (nring <= coarse size / 2, nangle >= 5, 1 <= c1, c2 <= 32)");
    if (b->is2d) return fail(GBR_ERR_UNSUPPORTED, "gbr_posenet_create: 2D classification has one direction");
    if ((size_t)desc->nring * desc->nangle * sizeof(float) > 48 * 1024 || b->ND > 8192)
        return fail(GBR_ERR_UNSUPPORTED, "gbr_posenet_create: nring x nangle <= 12288 bins, <= 8192 directions");
    std::unique_ptr<gbr_posenet> n(new gbr_posenet);
    n->b = b;
    n->seed = desc->seed;
    gbr::PnDims &d = n->d;
    d.B = desc->max_batch;
    d.H = desc->nring;
    d.W = desc->nangle;
    d.C1 = desc->c1;
    d.C2 = desc->c2;
    d.ND = (int)b->ND;
    const long long F = (long long)d.C2 * d.H;
    d.o_w1 = 0;
    d.o_b1 = d.o_w1 + (long long)d.C1 * 15;
    d.o_w2 = d.o_b1 + d.C1;
    d.o_b2 = d.o_w2 + (long long)d.C2 * d.C1 * 15;
    d.o_w3 = d.o_b2 + d.C2;
    d.o_b3 = d.o_w3 + F * d.ND;
    d.nparams = d.o_b3 + d.ND;
    n->nbins = d.H * d.W;
    // polar bin of every active coarse pixel: ring = shell, angle of (x, y) modulo pi
    const double kPi = 3.14159265358979323846;
    std::vector<int> bin(b->nc, -1);
    std::vector<int> cnt(n->nbins, 0);
    for (int j = 0; j < b->nc; ++j) {
        const PixelRef &pr = b->pc_h[j];
        if (pr.shell < 1 || pr.shell > d.H) continue;
        const double a = std::atan2((double)pr.y, (double)pr.x) + 0.5 * kPi;  // [0, pi]
        int t = (int)std::floor(a / kPi * d.W);
        if (t >= d.W) t -= d.W;
        if (t < 0) t = 0;
        bin[j] = (pr.shell - 1) * d.W + t;
        cnt[bin[j]] += 1;
    }
    std::vector<float> inv(n->nbins);
    for (int k = 0; k < n->nbins; ++k) inv[k] = cnt[k] ? 1.f / (float)cnt[k] : 0.f;
    GBR_CUDA(n->bin.upload(bin.data(), bin.size()));
    GBR_CUDA(n->inv_cnt.upload(inv.data(), inv.size()));
    // He-uniform initial weights, zero biases
    std::vector<float> p(d.nparams, 0.f);
    uint64_t z = host_mix64(desc->seed ^ 0x5EEDull);
    auto fill = [&](long long off, long long count, double fan_in) {
        const double a = std::sqrt(6.0 / fan_in);
        for (long long i = 0; i < count; ++i) {
            z = host_mix64(z);
            p[off + i] = (float)(a * (2.0 * ((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 1.0));
        }
    };
    fill(d.o_w1, (long long)d.C1 * 15, 15.0);
    fill(d.o_w2, (long long)d.C2 * d.C1 * 15, 15.0 * d.C1);
    fill(d.o_w3, F * d.ND, (double)F);
    GBR_CUDA(n->params.upload(p.data(), p.size()));
    GBR_CUDA(n->grad.reserve(d.nparams));
    GBR_CUDA(n->bw_scratch.reserve(gbr::pn_backward_scratch(d)));
    GBR_CUDA(n->m.reserve(d.nparams));
    GBR_CUDA(n->v.reserve(d.nparams));
    GBR_CUDA(n->m.zero());
    GBR_CUDA(n->v.zero());
    const size_t B = (size_t)d.B;
    GBR_CUDA(n->pw.reserve(B * b->nc));
    GBR_CUDA(n->feat.reserve(B * n->nbins));
    GBR_CUDA(n->a1.reserve(B * d.C1 * n->nbins));
    GBR_CUDA(n->d1.reserve(B * d.C1 * n->nbins));
    GBR_CUDA(n->a2.reserve(B * d.C2 * n->nbins));
    GBR_CUDA(n->d2.reserve(B * d.C2 * n->nbins));
    GBR_CUDA(n->h.reserve(B * F));
    GBR_CUDA(n->logits.reserve(B * d.ND));
    GBR_CUDA(n->dl.reserve(B * d.ND));
    GBR_CUDA(n->target.reserve(B * d.ND));
    GBR_CUDA(n->loss.reserve(B));
    GBR_CUDA(n->label.reserve(B));
    GBR_CUDA(n->fimg.reserve(B * b->full_npix));
    GBR_CUDA(cudaStreamCreateWithFlags(&n->st, cudaStreamNonBlocking));
    GBR_CUDA(cudaDeviceSynchronize());
    *out = n.release();
    return GBR_OK;
}

int gbr_posenet_destroy(gbr_posenet *n) {
    if (!n) return GBR_OK;
    cudaSetDevice(n->b->device);
    if (n->st) cudaStreamSynchronize(n->st);
    delete n;
    return GBR_OK;
}

int gbr_posenet_sizes(const gbr_posenet *n, int64_t *nparams, int64_t *nfeat, int64_t *ndir, int64_t *npix) {
    if (!n) return fail(GBR_ERR_INVALID, "null network");
    if (nparams) *nparams = n->d.nparams;
    if (nfeat) *nfeat = n->nbins;
    if (ndir) *ndir = n->d.ND;
    if (npix) *npix = n->b->nc;
    return GBR_OK;
}

int gbr_posenet_pixels(const gbr_posenet *n, int32_t *xy, float *minv) {
    if (!n || !xy || !minv) return fail(GBR_ERR_INVALID, "null argument");
    const gbr_bundle *b = n->b;
    for (int j = 0; j < b->nc; ++j) {
        xy[2 * j] = b->pc_h[j].x;
        xy[2 * j + 1] = b->pc_h[j].y;
    }
    GBR_CUDA(cudaSetDevice(b->device));
    GBR_CUDA(cudaMemcpy(minv, b->minv_c.p, sizeof(float) * b->nc, cudaMemcpyDeviceToHost));
    return GBR_OK;
}

int gbr_posenet_get_params(const gbr_posenet *n, float *out) {
    if (!n || !out) return fail(GBR_ERR_INVALID, "null argument");
    GBR_CUDA(cudaSetDevice(n->b->device));
    GBR_CUDA(cudaStreamSynchronize(n->st));
    GBR_CUDA(cudaMemcpy(out, n->params.p, sizeof(float) * n->d.nparams, cudaMemcpyDeviceToHost));
    return GBR_OK;
}

int gbr_posenet_set_params(gbr_posenet *n, const float *in) {
    if (!n || !in) return fail(GBR_ERR_INVALID, "null argument");
    GBR_CUDA(cudaSetDevice(n->b->device));
    GBR_CUDA(cudaStreamSynchronize(n->st));
    GBR_CUDA(cudaMemcpy(n->params.p, in, sizeof(float) * n->d.nparams, cudaMemcpyHostToDevice));
    return GBR_OK;
}

int gbr_posenet_features(gbr_posenet *n, const float *fimg, int64_t count, float *feat_out) {
    if (!n || (count > 0 && (!fimg || !feat_out))) return fail(GBR_ERR_INVALID, "null argument");
    GBR_CUDA(cudaSetDevice(n->b->device));
    const size_t full = (size_t)n->b->full_npix;
    for (int64_t c0 = 0; c0 < count; c0 += n->d.B) {
        const int c = (int)std::min<int64_t>(n->d.B, count - c0);
        int s = pn_features_dev(n, fimg + 2 * full * c0, c);
        if (s) return s;
        GBR_CUDA(cudaMemcpyAsync(feat_out + (size_t)n->nbins * c0, n->feat.p, sizeof(float) * n->nbins * c,
                                 cudaMemcpyDeviceToHost, n->st));
        GBR_CUDA(cudaStreamSynchronize(n->st));
    }
    return GBR_OK;
}

int gbr_posenet_loss_grad(gbr_posenet *n, const float *feat, const float *target, int64_t count, double *loss,
                          float *grad_out) {
    if (!n || !feat || !target || !loss || !grad_out) return fail(GBR_ERR_INVALID, "null argument");
    if (count < 1 || count > n->d.B) return fail(GBR_ERR_INVALID, "gbr_posenet_loss_grad: 1 <= count <= max_batch");
    GBR_CUDA(cudaSetDevice(n->b->device));
    gbr::PnDims d = n->d;
    d.B = (int)count;
    GBR_CUDA(cudaMemcpyAsync(n->feat.p, feat, sizeof(float) * n->nbins * count, cudaMemcpyHostToDevice, n->st));
    GBR_CUDA(cudaMemcpyAsync(n->target.p, target, sizeof(float) * d.ND * count, cudaMemcpyHostToDevice, n->st));
    GBR_CUDA(gbr::pn_forward(d, n->params.p, n->feat.p, n->a1.p, n->a2.p, n->h.p, n->logits.p, n->st));
    GBR_CUDA(gbr::pn_loss_backward(d, n->params.p, n->feat.p, n->a1.p, n->a2.p, n->h.p, n->logits.p, nullptr,
                                   n->target.p, n->dl.p, n->loss.p, n->d2.p, n->d1.p, n->grad.p, n->bw_scratch.p, n->st));
    std::vector<float> ls(count);
    GBR_CUDA(cudaMemcpyAsync(ls.data(), n->loss.p, sizeof(float) * count, cudaMemcpyDeviceToHost, n->st));
    GBR_CUDA(cudaMemcpyAsync(grad_out, n->grad.p, sizeof(float) * d.nparams, cudaMemcpyDeviceToHost, n->st));
    GBR_CUDA(cudaStreamSynchronize(n->st));
    double sum = 0.;
    for (float x : ls) sum += x;
    *loss = sum / (double)count;
    return GBR_OK;
}

int gbr_posenet_train(gbr_posenet *n, const float *ctf_pool, int64_t n_pool, int64_t steps, int64_t batch,
                      double lr, double *loss_out) {
    if (!n || !ctf_pool || n_pool < 1) return fail(GBR_ERR_INVALID, "null argument or empty CTF pool");
    if (batch < 1 || batch > n->d.B) return fail(GBR_ERR_INVALID, "gbr_posenet_train: 1 <= batch <= max_batch");
    if (steps < 0 || !(lr > 0.)) return fail(GBR_ERR_INVALID, "gbr_posenet_train: steps >= 0, lr > 0");
    gbr_bundle *b = n->b;
    GBR_CUDA(cudaSetDevice(b->device));
    const size_t full = (size_t)b->full_npix;
    GBR_CUDA(n->ctf_pool.reserve((size_t)n_pool * full));
    GBR_CUDA(cudaMemcpyAsync(n->ctf_pool.p, ctf_pool, sizeof(float) * full * n_pool, cudaMemcpyHostToDevice, n->st));
    gbr::PnDims d = n->d;
    d.B = (int)batch;
    std::vector<float> ls(batch);
    double acc = 0.;
    long long nacc = 0;
    for (int64_t k = 0; k < steps; ++k) {
        ++n->t;
        const uint64_t sd = host_mix64(n->seed ^ host_mix64((uint64_t)n->t));
        GBR_CUDA(gbr::pn_gen(b->proj_c.p, b->lda_c, b->pc.p, b->nc, b->minv_c.p, n->ctf_pool.p, (int)full,
                             (int)n_pool, b->R, (int)b->NP, (int)b->ND, sd, d.B, n->pw.p, n->label.p, n->st));
        GBR_CUDA(gbr::pn_bin(n->pw.p, b->nc, n->bin.p, n->inv_cnt.p, n->nbins, d.B, n->feat.p, n->st));
        GBR_CUDA(gbr::pn_forward(d, n->params.p, n->feat.p, n->a1.p, n->a2.p, n->h.p, n->logits.p, n->st));
        GBR_CUDA(gbr::pn_loss_backward(d, n->params.p, n->feat.p, n->a1.p, n->a2.p, n->h.p, n->logits.p,
                                       n->label.p, nullptr, n->dl.p, n->loss.p, n->d2.p, n->d1.p, n->grad.p,
                                       n->bw_scratch.p, n->st));
        GBR_CUDA(gbr::pn_adam(n->params.p, n->grad.p, n->m.p, n->v.p, d.nparams, (float)lr, (int)n->t, n->st));
        if (k >= steps - 20) {
            GBR_CUDA(cudaMemcpyAsync(ls.data(), n->loss.p, sizeof(float) * batch, cudaMemcpyDeviceToHost, n->st));
            GBR_CUDA(cudaStreamSynchronize(n->st));
            for (float x : ls) acc += x;
            nacc += batch;
        }
    }
    GBR_CUDA(cudaStreamSynchronize(n->st));
    if (loss_out) *loss_out = nacc ? acc / (double)nacc : 0.;
    return GBR_OK;
}

int gbr_posenet_train_targets(gbr_posenet *n, const float *fimg, const float *target, int64_t count, int64_t steps,
                              int64_t batch, double lr, double *loss_out) {
    if (!n || !fimg || !target || count < 1) return fail(GBR_ERR_INVALID, "null argument or empty particle set");
    if (batch < 1 || batch > n->d.B || batch > count)
        return fail(GBR_ERR_INVALID, "gbr_posenet_train_targets: 1 <= batch <= min(max_batch, count)");
    if (steps < 0 || !(lr > 0.)) return fail(GBR_ERR_INVALID, "gbr_posenet_train_targets: steps >= 0, lr > 0");
    gbr_bundle *b = n->b;
    GBR_CUDA(cudaSetDevice(b->device));
    const size_t full = (size_t)b->full_npix;
    const int nb = n->nbins, ND = n->d.ND;
    // features of every particle once, then targets; mini-batches are
    // consecutive windows of the set, cycling
    GBR_CUDA(n->feat_all.reserve((size_t)count * nb));
    GBR_CUDA(n->target_all.reserve((size_t)count * ND));
    for (int64_t c0 = 0; c0 < count; c0 += n->d.B) {
        const int c = (int)std::min<int64_t>(n->d.B, count - c0);
        int s = pn_features_dev(n, fimg + 2 * full * c0, c);
        if (s) return s;
        GBR_CUDA(cudaMemcpyAsync(n->feat_all.p + (size_t)nb * c0, n->feat.p, sizeof(float) * nb * c,
                                 cudaMemcpyDeviceToDevice, n->st));
    }
    GBR_CUDA(cudaMemcpyAsync(n->target_all.p, target, sizeof(float) * ND * count, cudaMemcpyHostToDevice, n->st));
    gbr::PnDims d = n->d;
    d.B = (int)batch;
    std::vector<float> ls(batch);
    double acc = 0.;
    long long nacc = 0;
    const int64_t nwin = count - batch + 1;
    for (int64_t k = 0; k < steps; ++k) {
        ++n->t;
        const int64_t s0 = (k * batch) % nwin;
        const float *f = n->feat_all.p + (size_t)nb * s0;
        const float *tg = n->target_all.p + (size_t)ND * s0;
        GBR_CUDA(gbr::pn_forward(d, n->params.p, f, n->a1.p, n->a2.p, n->h.p, n->logits.p, n->st));
        GBR_CUDA(gbr::pn_loss_backward(d, n->params.p, f, n->a1.p, n->a2.p, n->h.p, n->logits.p, nullptr, tg,
                                       n->dl.p, n->loss.p, n->d2.p, n->d1.p, n->grad.p, n->bw_scratch.p, n->st));
        GBR_CUDA(gbr::pn_adam(n->params.p, n->grad.p, n->m.p, n->v.p, d.nparams, (float)lr, (int)n->t, n->st));
        if (k >= steps - 20) {
            GBR_CUDA(cudaMemcpyAsync(ls.data(), n->loss.p, sizeof(float) * batch, cudaMemcpyDeviceToHost, n->st));
            GBR_CUDA(cudaStreamSynchronize(n->st));
            for (float x : ls) acc += x;
            nacc += batch;
        }
    }
    GBR_CUDA(cudaStreamSynchronize(n->st));
    if (loss_out) *loss_out = nacc ? acc / (double)nacc : 0.;
    return GBR_OK;
}

int gbr_posenet_block_probs(gbr_posenet *n, const float *fimg, int64_t count, int64_t dirs_per_block,
                            double temperature, float *out) {
    if (!n || (count > 0 && (!fimg || !out))) return fail(GBR_ERR_INVALID, "null argument");
    if (dirs_per_block < 1 || n->d.ND % dirs_per_block != 0 || !(temperature > 0.))
        return fail(GBR_ERR_INVALID, "gbr_posenet_block_probs: dirs_per_block must divide ndir, temperature > 0");
    GBR_CUDA(cudaSetDevice(n->b->device));
    const size_t full = (size_t)n->b->full_npix;
    const int nb = n->d.ND / (int)dirs_per_block;
    GBR_CUDA(n->prob.reserve((size_t)n->d.B * nb));
    for (int64_t c0 = 0; c0 < count; c0 += n->d.B) {
        const int c = (int)std::min<int64_t>(n->d.B, count - c0);
        int s = pn_features_dev(n, fimg + 2 * full * c0, c);
        if (s) return s;
        gbr::PnDims d = n->d;
        d.B = c;
        GBR_CUDA(gbr::pn_forward(d, n->params.p, n->feat.p, n->a1.p, n->a2.p, n->h.p, n->logits.p, n->st));
        GBR_CUDA(gbr::pn_block_probs(n->logits.p, d.ND, (int)dirs_per_block, (float)temperature, c, n->prob.p,
                                     n->st));
        GBR_CUDA(cudaMemcpyAsync(out + (size_t)nb * c0, n->prob.p, sizeof(float) * nb * c, cudaMemcpyDeviceToHost,
                                 n->st));
    }
    GBR_CUDA(cudaStreamSynchronize(n->st));
    return GBR_OK;
}

int gbr_posenet_propose_blocks(gbr_posenet *n, const float *fimg, int64_t count, int64_t dirs_per_block,
                               double temperature, int64_t m, int32_t *blocks_out, float *mass_out) {
    if (!n || (count > 0 && (!fimg || !blocks_out || !mass_out))) return fail(GBR_ERR_INVALID, "null argument");
    if (dirs_per_block < 1 || n->d.ND % dirs_per_block != 0 || !(temperature > 0.))
        return fail(GBR_ERR_INVALID, "gbr_posenet_propose_blocks: dirs_per_block must divide ndir, temperature > 0");
    const int nb = n->d.ND / (int)dirs_per_block;
    if (m < 1 || m > nb) return fail(GBR_ERR_INVALID, "gbr_posenet_propose_blocks: 1 <= m <= number of blocks");
    GBR_CUDA(cudaSetDevice(n->b->device));
    const size_t full = (size_t)n->b->full_npix;
    GBR_CUDA(n->prob.reserve((size_t)n->d.B * nb));
    GBR_CUDA(n->idx.reserve((size_t)n->d.B * m));
    GBR_CUDA(n->mass.reserve(n->d.B));
    for (int64_t c0 = 0; c0 < count; c0 += n->d.B) {
        const int c = (int)std::min<int64_t>(n->d.B, count - c0);
        int s = pn_features_dev(n, fimg + 2 * full * c0, c);
        if (s) return s;
        gbr::PnDims d = n->d;
        d.B = c;
        GBR_CUDA(gbr::pn_forward(d, n->params.p, n->feat.p, n->a1.p, n->a2.p, n->h.p, n->logits.p, n->st));
        GBR_CUDA(gbr::pn_block_probs(n->logits.p, d.ND, (int)dirs_per_block, (float)temperature, c, n->prob.p,
                                     n->st));
        GBR_CUDA(gbr::pn_top_blocks(n->prob.p, nb, (int)m, c, n->idx.p, n->mass.p, n->st));
        GBR_CUDA(cudaMemcpyAsync(blocks_out + m * c0, n->idx.p, sizeof(int32_t) * m * c, cudaMemcpyDeviceToHost,
                                 n->st));
        GBR_CUDA(cudaMemcpyAsync(mass_out + c0, n->mass.p, sizeof(float) * c, cudaMemcpyDeviceToHost, n->st));
    }
    GBR_CUDA(cudaStreamSynchronize(n->st));
    return GBR_OK;
}

int gbr_posenet_propose(gbr_posenet *n, const float *fimg, int64_t count, int64_t m, int32_t *dir_out,
                        float *prob_out) {
    if (!n || (count > 0 && (!fimg || !dir_out || !prob_out))) return fail(GBR_ERR_INVALID, "null argument");
    if (m < 1 || m > n->d.ND) return fail(GBR_ERR_INVALID, "gbr_posenet_propose: 1 <= m <= number of directions");
    GBR_CUDA(cudaSetDevice(n->b->device));
    const size_t full = (size_t)n->b->full_npix;
    GBR_CUDA(n->idx.reserve((size_t)n->d.B * m));
    GBR_CUDA(n->prob.reserve((size_t)n->d.B * m));
    for (int64_t c0 = 0; c0 < count; c0 += n->d.B) {
        const int c = (int)std::min<int64_t>(n->d.B, count - c0);
        int s = pn_features_dev(n, fimg + 2 * full * c0, c);
        if (s) return s;
        gbr::PnDims d = n->d;
        d.B = c;
        GBR_CUDA(gbr::pn_forward(d, n->params.p, n->feat.p, n->a1.p, n->a2.p, n->h.p, n->logits.p, n->st));
        GBR_CUDA(gbr::pn_topm(n->logits.p, d.ND, (int)m, c, n->idx.p, n->prob.p, n->st));
        GBR_CUDA(cudaMemcpyAsync(dir_out + m * c0, n->idx.p, sizeof(int32_t) * m * c, cudaMemcpyDeviceToHost, n->st));
        GBR_CUDA(cudaMemcpyAsync(prob_out + m * c0, n->prob.p, sizeof(float) * m * c, cudaMemcpyDeviceToHost, n->st));
        GBR_CUDA(cudaStreamSynchronize(n->st));
    }
    return GBR_OK;
}


}  // extern "C"
