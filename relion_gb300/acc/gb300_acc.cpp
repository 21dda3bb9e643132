// gb300_acc.cpp -- AccProjector, AccBackprojector, MlDeviceBundle and
// MlOptimiserCuda over libgbrelion's C ABI (the façade a relion_refine build
// links instead of src/acc/cuda/cuda_ml_optimiser.cu,
// src/acc/acc_projector_impl.h and src/acc/acc_backprojector_impl.h).
#include "cuda_ml_optimiser.h"

#include <algorithm>
#include <stdexcept>

void gbr_check(int st) {
    if (st != GBR_OK) {
        char msg[1024];
        gbr_last_error(msg, sizeof msg);
        throw std::runtime_error(std::string("libgbrelion: ") + msg);
    }
}

// ---- AccProjector -----------------------------------------------------------

bool AccProjector::setMdlDim(int xdim, int ydim, int zdim, int inity, int initz, int maxr, XFLOAT paddingFactor) {
    const bool changed = xdim != mdlX || ydim != mdlY || zdim != mdlZ || inity != mdlInitY || initz != mdlInitZ ||
                         maxr != mdlMaxR || paddingFactor != padding_factor;
    mdlX = xdim;
    mdlY = ydim;
    mdlZ = zdim;
    mdlInitY = inity;
    mdlInitZ = initz;
    mdlMaxR = maxr;
    padding_factor = paddingFactor;
    mdlXYZ = (size_t)xdim * ydim * zdim;
    return changed;
}

void AccProjector::initMdl(const XFLOAT *real, const XFLOAT *imag) {
    if (!bundle) throw std::runtime_error("AccProjector::initMdl: projector not attached to a bundle");
    std::vector<float> f(2 * mdlXYZ);
    for (size_t n = 0; n < mdlXYZ; ++n) {
        f[2 * n] = real[n];
        f[2 * n + 1] = imag[n];
    }
    gbr_check(gbr_projector_upload(bundle, iclass, f.data(), mdlX, mdlY, mdlZ, mdlInitY, mdlInitZ, mdlMaxR,
                                   (int64_t)padding_factor));
}

void AccProjector::initMdl(const Complex *data) {
    if (!bundle) throw std::runtime_error("AccProjector::initMdl: projector not attached to a bundle");
    std::vector<float> f(2 * mdlXYZ);
    for (size_t n = 0; n < mdlXYZ; ++n) {
        f[2 * n] = (float)data[n].real();
        f[2 * n + 1] = (float)data[n].imag();
    }
    gbr_check(gbr_projector_upload(bundle, iclass, f.data(), mdlX, mdlY, mdlZ, mdlInitY, mdlInitZ, mdlMaxR,
                                   (int64_t)padding_factor));
}

void AccProjector::clear() {
    // the device copy belongs to the bundle
    mdlX = mdlY = mdlZ = mdlMaxR = mdlInitY = mdlInitZ = 0;
    mdlXYZ = 0;
    bundle = nullptr;
}

// ---- AccBackprojector -------------------------------------------------------

size_t AccBackprojector::setMdlDim(int xdim, int ydim, int zdim, int inity, int initz, int max_r,
                                   XFLOAT paddingFactor) {
    if (!bundle) throw std::runtime_error("AccBackprojector::setMdlDim: not attached to a bundle");
    int64_t bx, by, bz, byi, bzi, br;
    gbr_check(gbr_backprojector_dims(bundle, &bx, &by, &bz, &byi, &bzi, &br));
    if (bx != xdim || by != ydim || bz != zdim || byi != inity || bzi != initz)
        throw std::runtime_error("AccBackprojector::setMdlDim: geometry differs from the bundle's volumes "
                                 "(sized from image_current_size)");
    mdlX = xdim;
    mdlY = ydim;
    mdlZ = zdim;
    mdlInitY = inity;
    mdlInitZ = initz;
    maxR = max_r;
    maxR2 = max_r * max_r;
    padding_factor = paddingFactor;
    mdlXYZ = (size_t)xdim * ydim * zdim;
    return mdlXYZ;
}

void AccBackprojector::initMdl() {
    if (!bundle) throw std::runtime_error("AccBackprojector::initMdl: not attached to a bundle");
    gbr_check(gbr_bundle_reset_wsum(bundle));
}

void AccBackprojector::getMdlData(double *real, double *imag, double *weights) {
    if (!bundle) throw std::runtime_error("AccBackprojector::getMdlData: not attached to a bundle");
    std::vector<double> d(2 * mdlXYZ);
    gbr_check(gbr_backprojector_download(bundle, iclass, d.data(), weights));
    for (size_t n = 0; n < mdlXYZ; ++n) {
        real[n] = d[2 * n];
        imag[n] = d[2 * n + 1];
    }
}

void AccBackprojector::getMdlData(XFLOAT *real, XFLOAT *imag, XFLOAT *weights) {
    std::vector<double> r(mdlXYZ), i(mdlXYZ), w(mdlXYZ);
    getMdlData(r.data(), i.data(), w.data());
    for (size_t n = 0; n < mdlXYZ; ++n) {
        real[n] = (XFLOAT)r[n];
        imag[n] = (XFLOAT)i[n];
        weights[n] = (XFLOAT)w[n];
    }
}

void AccBackprojector::clear() {
    mdlX = mdlY = mdlZ = mdlInitY = mdlInitZ = maxR = maxR2 = 0;
    mdlXYZ = 0;
    bundle = nullptr;
}

// ---- MlDeviceBundle ---------------------------------------------------------

void MlDeviceBundle::setupFixedSizedObjects() {
    MlOptimiser &o = *baseMLO;
    MlModel &m = o.mymodel;
    if (device_id < 0) throw std::runtime_error("MlDeviceBundle: setDevice() first");
    if (m.nr_classes < 1 || (int)m.PPref.size() != m.nr_classes)
        throw std::runtime_error("MlDeviceBundle: mymodel.PPref must hold nr_classes references");
    if (o.image_current_size.empty() || o.image_coarse_size.empty() || m.sigma2_noise.empty())
        throw std::runtime_error("MlDeviceBundle: image sizes and sigma2_noise of optics group 0 needed");
    projectors.clear();
    backprojectors.clear();
    if (handle) {
        gbr_bundle_destroy(handle);
        handle = nullptr;
    }
    gbr_model_desc d = {};
    d.ori_size = m.ori_size;
    d.nr_classes = m.nr_classes;
    d.current_size = o.image_current_size[0];
    d.coarse_size = o.image_coarse_size[0];
    d.padding_factor = m.padding_factor;
    d.healpix_order = o.sampling.healpix_order;
    d.adaptive_oversampling = o.adaptive_oversampling;
    d.maximum_significants = o.maximum_significants;
    d.sigma2_len = (int64_t)m.sigma2_noise[0].size();
    d.do_scale_correction = o.do_scale_correction;
    d.do_norm_correction = o.do_norm_correction;
    d.do_map = o.do_map;
    d.precision = precision;
    d.ref_dim = m.ref_dim;
    d.pixel_size = m.pixel_size;
    d.psi_step = o.sampling.psi_step;
    d.offset_range = o.sampling.offset_range;
    d.offset_step = o.sampling.offset_step;
    d.adaptive_fraction = o.adaptive_fraction;
    d.sigma2_fudge = o.sigma2_fudge;
    d.sigma2_offset = m.sigma2_offset;
    d.avg_norm_correction = m.avg_norm_correction;
    gbr_check(gbr_bundle_create(&d, device_id, &handle));

    projectors.resize(m.nr_classes);
    backprojectors.resize(m.nr_classes);
    int64_t bx, by, bz, byi, bzi, br;
    gbr_check(gbr_backprojector_dims(handle, &bx, &by, &bz, &byi, &bzi, &br));
    for (int i = 0; i < m.nr_classes; ++i) {
        const Projector &P = m.PPref[i];
        projectors[i].attach(handle, i);
        projectors[i].setMdlDim((int)P.xdim, (int)P.ydim, (int)P.zdim, (int)P.yinit, (int)P.zinit, P.r_max,
                                (XFLOAT)P.padding_factor);
        projectors[i].initMdl(P.data.data());
        backprojectors[i].attach(handle, i);
        backprojectors[i].setMdlDim((int)bx, (int)by, (int)bz, (int)byi, (int)bzi, (int)br,
                                    (XFLOAT)m.padding_factor);
    }
    std::vector<double> pdir;
    for (const std::vector<double> &row : m.pdf_direction) pdir.insert(pdir.end(), row.begin(), row.end());
    std::vector<double> dvp;
    for (const std::vector<double> &row : m.data_vs_prior_class) dvp.insert(dvp.end(), row.begin(), row.end());
    gbr_check(gbr_model_set_arrays(handle, m.sigma2_noise[0].data(), m.pdf_class.data(), pdir.data(),
                                   dvp.empty() ? nullptr : dvp.data()));
    gbr_optics_desc od = {};
    od.kV = o.obsModel.kV;
    od.Cs = o.obsModel.Cs;
    od.Q0 = o.obsModel.Q0;
    od.particle_diameter = o.particle_diameter;
    od.width_mask_edge = o.width_mask_edge;
    gbr_check(gbr_bundle_set_optics(handle, &od));
}

void MlDeviceBundle::setupTunableSizedObjects(size_t allocationSize) {
    if (!handle) throw std::runtime_error("MlDeviceBundle: setupFixedSizedObjects() first");
    gbr_check(gbr_bundle_reserve(handle, allocationSize));
}

void MlDeviceBundle::storeWeightedSumsIntoModel() {
    if (!handle) throw std::runtime_error("MlDeviceBundle: setupFixedSizedObjects() first");
    MlOptimiser &o = *baseMLO;
    MlWsumModel &w = o.wsum_model;
    const int K = o.mymodel.nr_classes;
    const size_t half = (size_t)o.mymodel.ori_size / 2 + 1;
    const size_t ndir = o.mymodel.pdf_direction.empty() ? 0 : o.mymodel.pdf_direction[0].size();
    std::vector<double> s2(half, 0.0), pcls(K, 0.0), pdir((size_t)K * ndir, 0.0);
    gbr_wsum ws = {};
    ws.sigma2_noise = s2.data();
    ws.pdf_class = pcls.data();
    ws.pdf_direction = pdir.data();
    gbr_check(gbr_wsum_download(handle, &ws));
    if (w.sigma2_noise.empty()) w.sigma2_noise.assign(1, std::vector<double>(half, 0.0));
    w.sigma2_noise[0].resize(half, 0.0);
    for (size_t i = 0; i < half; ++i) w.sigma2_noise[0][i] += s2[i];
    w.pdf_class.resize(K, 0.0);
    w.pdf_direction.resize(K);
    for (int k = 0; k < K; ++k) {
        w.pdf_class[k] += pcls[k];
        w.pdf_direction[k].resize(ndir, 0.0);
        for (size_t j = 0; j < ndir; ++j) w.pdf_direction[k][j] += pdir[(size_t)k * ndir + j];
    }
    w.sigma2_offset += ws.sigma2_offset;
    w.LL += ws.LL;
    w.ave_Pmax += ws.ave_Pmax;
    w.avg_norm_correction += ws.avg_norm_correction;
    if (w.sumw_group.empty()) w.sumw_group.assign(1, 0.0);
    w.sumw_group[0] += ws.sumw_group;

    w.BPref.resize(K);
    for (int k = 0; k < K; ++k) {
        AccBackprojector &A = backprojectors[k];
        BackProjector &B = w.BPref[k];
        if (B.data.size() != A.mdlXYZ) {
            B.data.assign(A.mdlXYZ, Complex(0.0, 0.0));
            B.weight.assign(A.mdlXYZ, 0.0);
            B.xdim = A.mdlX;
            B.ydim = A.mdlY;
            B.zdim = A.mdlZ;
            B.yinit = A.mdlInitY;
            B.zinit = A.mdlInitZ;
            B.r_max = A.maxR;
            B.padding_factor = (int)A.padding_factor;
        }
        std::vector<double> re(A.mdlXYZ), im(A.mdlXYZ), wt(A.mdlXYZ);
        A.getMdlData(re.data(), im.data(), wt.data());
        for (size_t n = 0; n < A.mdlXYZ; ++n) {
            B.data[n] += Complex(re[n], im[n]);
            B.weight[n] += wt[n];
        }
    }
}

MlDeviceBundle::~MlDeviceBundle() {
    projectors.clear();
    backprojectors.clear();
    if (handle) gbr_bundle_destroy(handle);
}

// ---- MlOptimiserCuda --------------------------------------------------------

MlOptimiserCuda::MlOptimiserCuda(MlOptimiser *baseMLOptimiser, MlDeviceBundle *b, const char *)
    : baseMLO(baseMLOptimiser), bundle(b), device_id(b->device_id),
      refIs3D(baseMLOptimiser->mymodel.ref_dim == 3), dataIs3D(baseMLOptimiser->mymodel.data_dim == 3) {
    if (!b->handle) throw std::runtime_error("MlOptimiserCuda: bundle not set up");
    gbr_check(gbr_worker_create(b->handle, &worker));
}

MlOptimiserCuda::~MlOptimiserCuda() {
    if (worker) gbr_worker_destroy(worker);
}

// First and last (inclusive) of n items for rank r of `size` (divide_equally,
// src/parallel.cpp).
static void share_of(long n, int size, int r, long &first, long &last) {
    const long base = n / size, rest = n % size;
    first = r * base + std::min<long>(r, rest);
    last = first + base + (r < rest ? 1 : 0) - 1;
}

void MlOptimiserCuda::doThreadExpectationSomeParticles(int thread_id) {
    MlOptimiser &o = *baseMLO;
    const long nbatch = o.exp_my_last_part_id - o.exp_my_first_part_id + 1;
    if (nbatch <= 0) return;
    if ((long)o.exp_imgs.size() != nbatch || (long)o.exp_metadata.size() != nbatch)
        throw std::runtime_error("MlOptimiserCuda: exp_imgs / exp_metadata must hold the batch's particles");
    if (thread_id < 0 || thread_id >= std::max(1, o.nr_threads))
        throw std::runtime_error("MlOptimiserCuda: thread_id outside nr_threads");
    long first, last;
    share_of(nbatch, std::max(1, o.nr_threads), thread_id, first, last);
    const long n = last - first + 1;
    if (n <= 0) return;
    const size_t npix = (size_t)o.mymodel.ori_size * o.mymodel.ori_size;
    std::vector<float> images(n * npix);
    std::vector<double> old_offset(2 * n), prior(2 * n), norm(n), scale(n), ctf(6 * n);
    const double sc = o.mymodel.scale_correction.empty() ? 1.0 : o.mymodel.scale_correction[0];
    for (long i = 0; i < n; ++i) {
        const std::vector<float> &img = o.exp_imgs[first + i];
        if (img.size() != npix) throw std::runtime_error("MlOptimiserCuda: image of the wrong size");
        std::copy(img.begin(), img.end(), images.begin() + i * npix);
        const std::vector<double> &md = o.exp_metadata[first + i];
        if (md.size() < (size_t)METADATA_LINE_LENGTH)
            throw std::runtime_error("MlOptimiserCuda: exp_metadata rows need METADATA_LINE_LENGTH columns");
        old_offset[2 * i] = md[METADATA_XOFF];
        old_offset[2 * i + 1] = md[METADATA_YOFF];
        prior[2 * i] = md[METADATA_XOFF_PRIOR];
        prior[2 * i + 1] = md[METADATA_YOFF_PRIOR];
        norm[i] = md[METADATA_NORM];
        scale[i] = sc;
        const int cols[6] = {METADATA_CTF_DEFOCUS_U, METADATA_CTF_DEFOCUS_V, METADATA_CTF_DEFOCUS_ANGLE,
                             METADATA_CTF_BFACTOR, METADATA_CTF_KFACTOR, METADATA_CTF_PHASE_SHIFT};
        for (int c = 0; c < 6; ++c) ctf[6 * i + c] = md[cols[c]];
    }
    gbr_image_batch in = {};
    in.n = n;
    in.device_resident = 0;
    in.images = images.data();
    in.old_offset = old_offset.data();
    in.prior = prior.data();
    in.norm_correction = norm.data();
    in.scale = scale.data();
    in.ctf = ctf.data();
    std::vector<gbr_particle_result> res(n);
    gbr_check(gbr_expect_images(worker, &in, res.data()));
    for (long i = 0; i < n; ++i) {
        std::vector<double> &md = o.exp_metadata[first + i];
        const gbr_particle_result &r = res[i];
        md[METADATA_ROT] = r.rot;
        md[METADATA_TILT] = r.tilt;
        md[METADATA_PSI] = r.psi;
        md[METADATA_XOFF] = r.xoff;
        md[METADATA_YOFF] = r.yoff;
        md[METADATA_CLASS] = r.cls;
        md[METADATA_DLL] = r.dLL;
        md[METADATA_PMAX] = r.pmax;
        md[METADATA_NR_SIGN] = r.nr_sign;
        md[METADATA_NORM] = r.norm;
    }
}
