// facade_estep.cpp -- test driver of the C++ façade (relion_gb300/acc).
//
//   facade_estep --version         print gbr_version() (no device work)
//   facade_estep REQUEST RESPONSE  one E-step batch through MlDeviceBundle /
//                                  MlOptimiserCuda, one worker per thread
//
// REQUEST and RESPONSE are flat float64 files; their layouts are written by
// and read in tests/test_gpu_facade.py (_request, _response).
#include <cstdio>
#include <cstring>
#include <exception>
#include <fstream>
#include <memory>
#include <vector>

#include "cuda_ml_optimiser.h"

namespace {

struct Reader {
    std::vector<double> v;
    size_t k = 0;
    double next() {
        if (k >= v.size()) throw std::runtime_error("request too short");
        return v[k++];
    }
    long inext() { return (long)next(); }
};

std::vector<double> read_all(const char *path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error(std::string("cannot open ") + path);
    f.seekg(0, std::ios::end);
    const size_t bytes = (size_t)f.tellg();
    f.seekg(0);
    std::vector<double> v(bytes / sizeof(double));
    f.read(reinterpret_cast<char *>(v.data()), (std::streamsize)(v.size() * sizeof(double)));
    return v;
}

int run(const char *req_path, const char *resp_path) {
    Reader r{read_all(req_path)};
    MlOptimiser o;
    MlModel &m = o.mymodel;
    m.ori_size = (int)r.inext();
    m.nr_classes = (int)r.inext();
    o.image_current_size = {(int)r.inext()};
    o.image_coarse_size = {(int)r.inext()};
    m.padding_factor = (int)r.inext();
    o.sampling.healpix_order = (int)r.inext();
    o.sampling.psi_step = r.next();
    o.sampling.offset_range = r.next();
    o.sampling.offset_step = r.next();
    m.pixel_size = r.next();
    o.adaptive_fraction = r.next();
    o.sigma2_fudge = r.next();
    m.sigma2_offset = r.next();
    m.avg_norm_correction = r.next();
    o.do_norm_correction = r.inext() != 0;
    o.do_scale_correction = r.inext() != 0;
    o.do_map = r.inext() != 0;
    o.maximum_significants = (int)r.inext();
    o.adaptive_oversampling = (int)r.inext();
    const int precision = (int)r.inext();
    const int device = (int)r.inext();
    o.nr_threads = (int)r.inext();
    const long n = r.inext();
    o.obsModel.kV = r.next();
    o.obsModel.Cs = r.next();
    o.obsModel.Q0 = r.next();
    o.particle_diameter = r.next();
    o.width_mask_edge = r.next();
    m.scale_correction = {r.next()};
    m.ref_dim = (int)r.inext();
    m.PPref.resize(m.nr_classes);
    for (Projector &P : m.PPref) {
        P.xdim = r.inext();
        P.ydim = r.inext();
        P.zdim = r.inext();
        P.yinit = r.inext();
        P.zinit = r.inext();
        P.r_max = (int)r.inext();
        P.padding_factor = (int)r.inext();
        P.data.resize((size_t)P.xdim * P.ydim * P.zdim);
        for (Complex &c : P.data) {
            const double re = r.next();
            c = Complex(re, r.next());
        }
    }
    const size_t half = (size_t)m.ori_size / 2 + 1;
    m.sigma2_noise.assign(1, std::vector<double>(half));
    for (double &x : m.sigma2_noise[0]) x = r.next();
    m.pdf_class.resize(m.nr_classes);
    for (double &x : m.pdf_class) x = r.next();
    const long ndir = r.inext();
    m.pdf_direction.assign(m.nr_classes, std::vector<double>(ndir));
    for (std::vector<double> &row : m.pdf_direction)
        for (double &x : row) x = r.next();
    o.exp_my_first_part_id = 0;
    o.exp_my_last_part_id = n - 1;
    const size_t npix = (size_t)m.ori_size * m.ori_size;
    o.exp_imgs.assign(n, std::vector<float>(npix));
    o.exp_metadata.assign(n, std::vector<double>(METADATA_LINE_LENGTH, 0.0));
    for (long i = 0; i < n; ++i) {
        for (float &x : o.exp_imgs[i]) x = (float)r.next();
        for (double &x : o.exp_metadata[i]) x = r.next();
    }

    MlDeviceBundle bundle(&o);
    bundle.precision = precision;
    bundle.setDevice(device);
    bundle.setupFixedSizedObjects();
    bundle.setupTunableSizedObjects((size_t)4 << 30);
    {
        std::vector<std::unique_ptr<MlOptimiserCuda>> threads;
        for (int t = 0; t < o.nr_threads; ++t) threads.emplace_back(new MlOptimiserCuda(&o, &bundle, ""));
        for (int t = 0; t < o.nr_threads; ++t) {
            threads[t]->resetData();
            threads[t]->doThreadExpectationSomeParticles(t);
        }
    }
    bundle.syncAllBackprojects();
    bundle.storeWeightedSumsIntoModel();

    std::vector<double> out;
    for (const std::vector<double> &row : o.exp_metadata) out.insert(out.end(), row.begin(), row.end());
    const MlWsumModel &w = o.wsum_model;
    out.insert(out.end(), w.sigma2_noise[0].begin(), w.sigma2_noise[0].end());
    out.insert(out.end(), w.pdf_class.begin(), w.pdf_class.end());
    for (const std::vector<double> &row : w.pdf_direction) out.insert(out.end(), row.begin(), row.end());
    out.push_back(w.sigma2_offset);
    out.push_back(w.LL);
    out.push_back(w.ave_Pmax);
    out.push_back(w.avg_norm_correction);
    out.push_back(w.sumw_group[0]);
    for (const BackProjector &B : w.BPref) {
        out.push_back((double)B.xdim);
        out.push_back((double)B.ydim);
        out.push_back((double)B.zdim);
        for (const Complex &c : B.data) {
            out.push_back(c.real());
            out.push_back(c.imag());
        }
        out.insert(out.end(), B.weight.begin(), B.weight.end());
    }
    std::ofstream f(resp_path, std::ios::binary);
    f.write(reinterpret_cast<const char *>(out.data()), (std::streamsize)(out.size() * sizeof(double)));
    return f ? 0 : 1;
}

}  // namespace

int main(int argc, char **argv) {
    try {
        if (argc == 2 && std::strcmp(argv[1], "--version") == 0) {
            std::printf("%s\n", gbr_version());
            return 0;
        }
        if (argc != 3) {
            std::fprintf(stderr, "usage: facade_estep --version | REQUEST RESPONSE\n");
            return 2;
        }
        return run(argv[1], argv[2]);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "facade_estep: %s\n", e.what());
        return 1;
    }
}
