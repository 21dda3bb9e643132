// ml_optimiser_stub.h -- the members of RELION's MlOptimiser that the GB300
// E-step façade reads and writes, as plain C++ containers.
//
// Stand-in for src/ml_optimiser.h (class MlOptimiser), src/ml_model.h
// (MlModel, MlWsumModel), src/healpix_sampling.h (HealpixSampling),
// src/projector.h / src/backprojector.h (Projector, BackProjector) when the
// façade is compiled outside relion_refine.  Member names are the
// reference's, so the façade's code reads as it would against the real
// classes; the containers are std::vector instead of MultidimArray, complex
// values are std::complex<double> (RELION's Complex with RFLOAT = double) and
// offsets are in pixels.  Only the 2D-image, one-optics-group path is
// represented, as in the library.
#ifndef GB300_ML_OPTIMISER_STUB_H
#define GB300_ML_OPTIMISER_STUB_H

#include <complex>
#include <vector>

typedef std::complex<double> Complex;

// Columns of MlOptimiser::exp_metadata used by the E-step (the reference's
// METADATA_* column indices, src/ml_optimiser.h:51-79).
enum {
    METADATA_ROT = 0, METADATA_TILT = 1, METADATA_PSI = 2, METADATA_XOFF = 3, METADATA_YOFF = 4,
    METADATA_ZOFF = 5, METADATA_CLASS = 6, METADATA_DLL = 7, METADATA_PMAX = 8, METADATA_NR_SIGN = 9,
    METADATA_NORM = 10, METADATA_CTF_DEFOCUS_U = 11, METADATA_CTF_DEFOCUS_V = 12,
    METADATA_CTF_DEFOCUS_ANGLE = 13, METADATA_CTF_BFACTOR = 14, METADATA_CTF_KFACTOR = 15,
    METADATA_CTF_PHASE_SHIFT = 16, METADATA_ROT_PRIOR = 17, METADATA_TILT_PRIOR = 18,
    METADATA_PSI_PRIOR = 19, METADATA_XOFF_PRIOR = 20, METADATA_YOFF_PRIOR = 21,
    METADATA_ZOFF_PRIOR = 22, METADATA_PSI_PRIOR_FLIP_RATIO = 23, METADATA_ROT_PRIOR_FLIP_RATIO = 24,
    METADATA_LINE_LENGTH = 25
};

// Projector: padded Fourier-space reference [zdim][ydim][xdim] with logical
// origin (0, yinit, zinit) and the radius r_max of the data it holds.
struct Projector {
    std::vector<Complex> data;
    long xdim = 0, ydim = 0, zdim = 0, yinit = 0, zinit = 0;
    int r_max = 0, padding_factor = 2, ori_size = 0;
};

// BackProjector: accumulated data and weight volumes, same layout.
struct BackProjector {
    std::vector<Complex> data;
    std::vector<double> weight;
    long xdim = 0, ydim = 0, zdim = 0, yinit = 0, zinit = 0;
    int r_max = 0, padding_factor = 2;
};

struct MlModel {
    int ori_size = 0, nr_classes = 1, ref_dim = 3, data_dim = 2, padding_factor = 2;
    double pixel_size = 1.0, sigma2_offset = 0.0, avg_norm_correction = 1.0;
    std::vector<Projector> PPref;                        // [K]
    std::vector<std::vector<double>> sigma2_noise;       // [group][ori/2+1]
    std::vector<double> pdf_class;                       // [K]
    std::vector<std::vector<double>> pdf_direction;      // [K][ndir]
    std::vector<std::vector<double>> data_vs_prior_class;  // [K][ori/2+1] (scale correction only)
    std::vector<double> scale_correction;                // [group]
};

struct MlWsumModel {
    std::vector<BackProjector> BPref;                    // [K]
    std::vector<std::vector<double>> sigma2_noise;       // [group][ori/2+1]
    std::vector<double> pdf_class;                       // [K]
    std::vector<std::vector<double>> pdf_direction;      // [K][ndir]
    double sigma2_offset = 0.0, LL = 0.0, ave_Pmax = 0.0, avg_norm_correction = 0.0;
    std::vector<double> sumw_group;                      // [group]
};

struct HealpixSampling {
    int healpix_order = 2;
    double psi_step = -1.0, offset_range = 6.0, offset_step = 2.0;  // degrees, Angstrom
};

// Optics of the particles' (single) optics group (ObservationModel).
struct ObservationModel {
    double kV = 300.0, Cs = 2.7, Q0 = 0.1;
};

class MlOptimiser {
public:
    MlModel mymodel;
    MlWsumModel wsum_model;
    HealpixSampling sampling;
    ObservationModel obsModel;
    std::vector<int> image_current_size, image_coarse_size;  // [optics group]
    int adaptive_oversampling = 1, maximum_significants = -1;
    bool do_scale_correction = false, do_norm_correction = true, do_map = true;
    double adaptive_fraction = 0.999, sigma2_fudge = 1.0;
    double particle_diameter = -1.0, width_mask_edge = 5.0;
    int nr_threads = 1;

    // the particles of the current batch: part ids exp_my_first_part_id ..
    // exp_my_last_part_id (inclusive); row i of exp_imgs / exp_metadata is
    // particle exp_my_first_part_id + i
    long exp_my_first_part_id = 0, exp_my_last_part_id = -1;
    std::vector<std::vector<float>> exp_imgs;            // [i][ori*ori] real-space image
    std::vector<std::vector<double>> exp_metadata;       // [i][METADATA_LINE_LENGTH]
};

#endif
