// ref_estep_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's own CPU expectation step on given inputs: an
// MlOptimiser whose model, sampling, particle table and options are set
// from the request, then, per particle, the sequence of
// MlOptimiser::expectationOneParticle (src/ml_optimiser.cpp:4376-4700)
// after its image preparation: getAllSquaredDifferences (:7098) and
// convertAllSquaredDifferencesToWeights (:7704) for the coarse and the fine
// pass, then storeWeightedSums (:8241).  The prepared images (masked and
// unmasked Fourier transforms, CTF image, power spectrum, Xi2) are the
// request's, so that the oracle and the CUDA E-step can be compared with the
// reference on identical inputs.  Compiled by oracle/build_ref.sh with the
// reference's sources, where they lie; never part of the product.
//
//   ref_estep <request file> <response file>
//
// Request (float64): ori, cur, coarse, pad, healpix order, psi step (deg),
//   offset range (A), offset step (A), pixel size (A), adaptive fraction,
//   sigma2 fudge, sigma2_offset (A^2), n particles, projector xdim, ydim,
//   zdim, yinit, zinit, r_max; projector data (complex); sigma2_noise
//   [ori/2+1]; pdf_direction [ndir]; then per particle fimg, fimg_nomask
//   (complex [cur][cur/2+1]), fctf [cur][cur/2+1], power_img [ori/2+1],
//   old offset (x, y px), prior (x, y px), highres_Xi2, norm_correction.
// Response (float64): per particle the coarse pass (n, diff2 [n], weights
//   [n], significant [n]), the fine pass (n, diff2 [n], weights [n]), the
//   scalars coarse min diff2, coarse sum of weights, coarse significant
//   weight, fine min diff2, fine sum of weights, fine significant weight,
//   max weight, and the metadata row (rot, tilt, psi, xoff, yoff, class,
//   dLL, pmax, nr_sign, norm); then the weighted sums: sigma2_noise
//   [ori/2+1], pdf_class, pdf_direction [ndir], sigma2_offset, sumw_group,
//   LL, ave_Pmax, avg_norm_correction, backprojector xdim, ydim, zdim, data
//   (complex), weight.
#include "src/ml_optimiser.h"

#include <cstdio>
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

void read_complex(Reader &r, MultidimArray<Complex> &a) {
    for (long n = 0; n < (long)MULTIDIM_SIZE(a); ++n) {
        const double re = r.d(), im = r.d();
        a.data[n] = Complex(re, im);
    }
}

// Resolution shell of each pixel of a [size][size/2+1] transform (-1 outside
// size/2 and for the redundant half of the x = 0 column), as
// MlOptimiser::updateImageSizeAndResolutionPointers fills Mresol.
void fill_mresol(MultidimArray<int> &M, int size) {
    M.resize(size, size / 2 + 1);
    M.initConstant(-1);
    FOR_ALL_ELEMENTS_IN_FFTW_TRANSFORM2D(M) {
        const int ires = ROUND(sqrt((RFLOAT)(ip * ip + jp * jp)));
        if (ires < size / 2 + 1 && !(jp == 0 && ip < 0)) DIRECT_A2D_ELEM(M, i, j) = ires;
    }
}

void run(Reader &r, std::vector<double> &out) {
    const long ori = r.l(), cur = r.l(), crs = r.l(), pad = r.l(), order = r.l();
    const double psi_step = r.d(), orange = r.d(), ostep = r.d(), pix = r.d(), afrac = r.d(), fudge = r.d(),
                 s2off = r.d();
    const long n = r.l();
    const long xdim = r.l(), ydim = r.l(), zdim = r.l(), yinit = r.l(), zinit = r.l(), r_max = r.l();

    MlOptimiser o;
    // options of a plain relion_refine CPU run (no GPU, no helical / multi-body
    // / tomography, exact shifts, adaptive oversampling 1)
    o.do_gpu = o.do_cpu = o.do_sycl = false;
    o.do_grad = false;
    o.do_helical_refine = o.ignore_helical_symmetry = false;
    o.do_skip_align = o.do_skip_rotate = o.do_only_sample_tilt = false;
    o.do_skip_maximization = false;
    o.do_shifts_onthefly = false;
    o.do_firstiter_cc = o.do_always_cc = false;
    o.do_ctf_correction = true;
    o.refs_are_ctf_corrected = true;
    o.do_scale_correction = false;
    o.do_norm_correction = false;
    o.do_map = true;
    o.adaptive_oversampling = 1;
    o.adaptive_fraction = afrac;
    o.maximum_significants = -1;
    o.sigma2_fudge = fudge;
    o.strict_highres_exp = -1.;
    o.offset_range_x = o.offset_range_y = o.offset_range_z = -1.;  // --offset_range_x etc. not given
    o.iter = 2;

    // model
    MlModel &m = o.mymodel;
    m.ori_size = (int)ori;
    m.pixel_size = pix;
    m.current_size = (int)cur;
    m.nr_classes = 1;
    m.nr_bodies = 1;
    m.nr_groups = 1;
    m.nr_optics_groups = 1;
    m.ref_dim = 3;
    m.data_dim = 2;
    m.padding_factor = (RFLOAT)pad;
    m.interpolator = TRILINEAR;
    m.r_min_nn = 10;
    m.orientational_prior_mode = NOPRIOR;
    m.sigma2_offset = s2off;
    m.avg_norm_correction = 1.;
    m.ave_Pmax = 0.;
    m.LL = 0.;
    m.do_grad = false;
    m.pdf_class.assign(1, 1.);
    m.class_age.assign(1, 0.);
    m.is_helix = false;
    m.helical_nr_asu = 1;
    m.helical_twist.assign(1, 0.);
    m.helical_rise.assign(1, 0.);
    m.sigma2_rot = m.sigma2_tilt = m.sigma2_psi = 0.;
    m.scale_correction.assign(1, 1.);
    m.prior_offset_class.assign(1, Matrix1D<RFLOAT>(2));
    m.prior_offset_class[0].initZeros();
    m.PPref.assign(1, Projector((int)ori, TRILINEAR, (float)pad, 10, 2));
    Projector &P = m.PPref[0];
    P.r_max = (int)r_max;
    P.ref_dim = 3;
    P.pad_size = (int)ydim;
    P.data.resize(zdim, ydim, xdim);
    P.data.yinit = yinit;
    P.data.zinit = zinit;
    P.data.xinit = 0;
    read_complex(r, P.data);
    m.sigma2_noise.assign(1, MultidimArray<RFLOAT>(ori / 2 + 1));
    for (long k = 0; k < ori / 2 + 1; ++k) m.sigma2_noise[0].data[k] = r.d();
    m.data_vs_prior_class.assign(1, MultidimArray<RFLOAT>(ori / 2 + 1));
    m.data_vs_prior_class[0].initZeros();

    // sampling (C1)
    HealpixSampling &S = o.sampling;
    S.healpix_order = (int)order;
    S.psi_step = psi_step;
    S.offset_range = orange;
    S.offset_step = ostep;
    S.fn_sym = "C1";
    S.limit_tilt = -91.;
    S.initialise(3);
    S.random_perturbation = 0.;
    const long ndir = S.NrDirections();
    m.nr_directions = ndir;
    m.pdf_direction.assign(1, MultidimArray<RFLOAT>(ndir));
    for (long k = 0; k < ndir; ++k) m.pdf_direction[0].data[k] = r.d();

    // weighted sums (backprojector at the current size)
    o.wsum_model.initialise(m, "C1", false, true, false);
    o.wsum_model.current_size = (int)cur;
    o.wsum_model.initZeros();

    // particles: one optics group (pixel size, box), one group, one image each
    MetaDataTable opt;
    opt.setName("optics");
    opt.addObject();
    opt.setValue(EMDL_IMAGE_OPTICS_GROUP, 1);
    opt.setValue(EMDL_IMAGE_OPTICS_GROUP_NAME, std::string("opticsGroup1"));
    opt.setValue(EMDL_IMAGE_PIXEL_SIZE, pix);
    opt.setValue(EMDL_IMAGE_SIZE, (int)ori);
    opt.setValue(EMDL_IMAGE_DIMENSIONALITY, 2);
    opt.setValue(EMDL_CTF_VOLTAGE, 300.);
    opt.setValue(EMDL_CTF_CS, 2.7);
    opt.setValue(EMDL_CTF_Q0, 0.1);
    o.mydata.obsModel = ObservationModel(opt);
    o.mydata.is_tomo = false;
    o.mydata.nr_particles_per_optics_group.assign(1, 0);
    const long gid = o.mydata.addGroup("mic", 0);
    for (long p = 0; p < n; ++p) {
        o.mydata.addParticle("particle", 0, gid);
        o.mydata.addImageToParticle(p);
    }
    o.exp_my_first_part_id = 0;
    o.exp_my_last_part_id = n - 1;
    o.image_full_size.assign(1, (int)ori);
    o.image_current_size.assign(1, (int)cur);
    o.image_coarse_size.assign(1, (int)crs);
    o.Mresol_fine.resize(1);
    o.Mresol_coarse.resize(1);
    fill_mresol(o.Mresol_fine[0], (int)cur);
    fill_mresol(o.Mresol_coarse[0], (int)crs);
    o.exp_metadata.initZeros(n, METADATA_LINE_LENGTH_BEFORE_BODIES);
    for (long p = 0; p < n; ++p) DIRECT_A2D_ELEM(o.exp_metadata, p, METADATA_NORM) = 1.;

    const long X = cur / 2 + 1;
    for (long p = 0; p < n; ++p) {
        std::vector<MultidimArray<Complex>> Fimg(1, MultidimArray<Complex>(cur, X)), Fnm(1, MultidimArray<Complex>(cur, X));
        std::vector<MultidimArray<RFLOAT>> Fctf(1, MultidimArray<RFLOAT>(cur, X)), power(1, MultidimArray<RFLOAT>(ori / 2 + 1));
        read_complex(r, Fimg[0]);
        read_complex(r, Fnm[0]);
        for (long k = 0; k < (long)MULTIDIM_SIZE(Fctf[0]); ++k) Fctf[0].data[k] = r.d();
        for (long k = 0; k < ori / 2 + 1; ++k) power[0].data[k] = r.d();
        Matrix1D<RFLOAT> old_offset(2), prior(2);
        old_offset(0) = r.d();
        old_offset(1) = r.d();
        prior(0) = r.d();
        prior(1) = r.d();
        std::vector<RFLOAT> xi2(1, r.d());
        DIRECT_A2D_ELEM(o.exp_metadata, p, METADATA_NORM) = r.d();
        DIRECT_A2D_ELEM(o.exp_metadata, p, METADATA_XOFF) = old_offset(0);
        DIRECT_A2D_ELEM(o.exp_metadata, p, METADATA_YOFF) = old_offset(1);
        DIRECT_A2D_ELEM(o.exp_metadata, p, METADATA_XOFF_PRIOR) = prior(0);
        DIRECT_A2D_ELEM(o.exp_metadata, p, METADATA_YOFF_PRIOR) = prior(1);

        std::vector<std::vector<MultidimArray<Complex>>> sh, sh_nm;
        std::vector<MultidimArray<RFLOAT>> loc_ctf;
        std::vector<int> pdir, ppsi;
        std::vector<RFLOAT> dprior, pprior, sqrtxi2;
        MultidimArray<RFLOAT> Mw, minv, stmulti;
        MultidimArray<bool> sig;
        RFLOAT min_diff2 = 0., sum_w = 0., sig_w = -1., max_w = 0.;
        const int idir_max = (int)S.NrDirections(0, &pdir) - 1, ipsi_max = (int)S.NrPsiSamplings(0, &ppsi) - 1;
        const int itrans_max = (int)S.NrTranslationalSamplings() - 1;
        double c_min = 0., c_sum = 0., c_sig = 0.;
        for (int ipass = 0; ipass < 2; ++ipass) {
            const int ov = ipass == 0 ? 0 : 1;
            o.getAllSquaredDifferences(p, 0, ipass, ov, (int)p, 0, idir_max, 0, ipsi_max, 0, itrans_max, 0, 0,
                                       min_diff2, xi2, Fimg, Fctf, old_offset, Mw, sig, pdir, ppsi, dprior, pprior, sh,
                                       minv, loc_ctf, sqrtxi2, stmulti);
            out.push_back((double)MULTIDIM_SIZE(Mw));
            for (long k = 0; k < (long)MULTIDIM_SIZE(Mw); ++k) out.push_back(Mw.data[k]);
            o.convertAllSquaredDifferencesToWeights(p, 0, ipass, ov, (int)p, 0, idir_max, 0, ipsi_max, 0, itrans_max,
                                                    0, 0, Mw, sig, sig_w, sum_w, old_offset, prior, min_diff2, pdir,
                                                    ppsi, dprior, pprior);
            for (long k = 0; k < (long)MULTIDIM_SIZE(Mw); ++k) out.push_back(Mw.data[k]);
            if (ipass == 0) {
                for (long k = 0; k < (long)MULTIDIM_SIZE(Mw); ++k) out.push_back(DIRECT_A1D_ELEM(sig, k) ? 1. : 0.);
                c_min = min_diff2;
                c_sum = sum_w;
                c_sig = sig_w;
            }
        }
        o.storeWeightedSums(p, 0, 1, (int)p, 0, idir_max, 0, ipsi_max, 0, itrans_max, 0, 0, min_diff2, xi2, Fimg, Fnm,
                            Fctf, power, old_offset, prior, Mw, sig, sig_w, sum_w, max_w, pdir, ppsi, dprior, pprior,
                            sh, sh_nm, minv, loc_ctf, sqrtxi2, stmulti);
        for (double v : {c_min, c_sum, c_sig, (double)min_diff2, (double)sum_w, (double)sig_w, (double)max_w})
            out.push_back(v);
        for (int c : {METADATA_ROT, METADATA_TILT, METADATA_PSI, METADATA_XOFF, METADATA_YOFF, METADATA_CLASS,
                      METADATA_DLL, METADATA_PMAX, METADATA_NR_SIGN, METADATA_NORM})
            out.push_back(DIRECT_A2D_ELEM(o.exp_metadata, p, c));
    }
    MlWsumModel &w = o.wsum_model;
    for (long k = 0; k < ori / 2 + 1; ++k) out.push_back(w.sigma2_noise[0].data[k]);
    out.push_back(w.pdf_class[0]);
    for (long k = 0; k < ndir; ++k) out.push_back(w.pdf_direction[0].data[k]);
    out.push_back(w.sigma2_offset);
    out.push_back(w.sumw_group[0]);
    out.push_back(w.LL);
    out.push_back(w.ave_Pmax);
    out.push_back(w.avg_norm_correction);
    BackProjector &B = w.BPref[0];
    out.push_back(XSIZE(B.data));
    out.push_back(YSIZE(B.data));
    out.push_back(ZSIZE(B.data));
    for (long k = 0; k < (long)MULTIDIM_SIZE(B.data); ++k) {
        out.push_back(B.data.data[k].real);
        out.push_back(B.data.data[k].imag);
    }
    for (long k = 0; k < (long)MULTIDIM_SIZE(B.weight); ++k) out.push_back(B.weight.data[k]);
}

}  // namespace

int main(int argc, char **argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: ref_estep <request> <response>\n");
        return 2;
    }
    try {
        const std::vector<double> req = read_all(argv[1]);
        Reader r{req};
        std::vector<double> out;
        run(r, out);
        write_all(argv[2], out);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "ref_estep: %s\n", e.what());
        return 1;
    } catch (RelionError &e) {
        std::fprintf(stderr, "ref_estep: RelionError %s\n", e.msg.c_str());
        return 1;
    }
    return 0;
}
