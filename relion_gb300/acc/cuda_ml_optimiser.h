// cuda_ml_optimiser.h -- MlDeviceBundle and MlOptimiserCuda of the GB300
// façade: the reference's accelerated E-step classes
// (src/acc/cuda/cuda_ml_optimiser.h:18-146) over libgbrelion's C ABI, with
// the reference's constructors and member functions, so that MlOptimiser's
// dispatch (src/ml_optimiser.cpp:3570-3600, 78-97) drives them unchanged.
//
//   MlDeviceBundle b(&mlo);  b.setDevice(0);  b.setupFixedSizedObjects();
//   b.setupTunableSizedObjects(bytes);
//   MlOptimiserCuda w(&mlo, &b, "");         // one per thread
//   w.doThreadExpectationSomeParticles(t);   // thread t's share of the batch
//   b.syncAllBackprojects();  b.storeWeightedSumsIntoModel();
//
// Errors of the library raise std::runtime_error carrying gbr_last_error().
#ifndef GB300_CUDA_ML_OPTIMISER_H
#define GB300_CUDA_ML_OPTIMISER_H

#include <string>
#include <vector>

#include "acc_backprojector.h"
#include "acc_projector.h"
#include "gbrelion.h"
#include "ml_optimiser_stub.h"

// Throws std::runtime_error("libgbrelion: <last error>") unless st == GBR_OK.
void gbr_check(int st);

class MlDeviceBundle {
public:
    std::vector<AccProjector> projectors;        // one per class
    std::vector<AccBackprojector> backprojectors;
    MlOptimiser *baseMLO;
    int device_id = -1;
    int rank_shared_count = 1;
    // coarse-pass arithmetic (no counterpart in the reference):
    // GBR_PREC_BF16 tcgen05 precision form, GBR_PREC_FP32 plain path
    int precision = GBR_PREC_BF16;
    gbr_bundle *handle = nullptr;

    explicit MlDeviceBundle(MlOptimiser *baseMLOptimiser) : baseMLO(baseMLOptimiser) {}
    MlDeviceBundle(const MlDeviceBundle &) = delete;
    MlDeviceBundle &operator=(const MlDeviceBundle &) = delete;

    void setDevice(int did) { device_id = did; }

    // The iteration's model, sampling and references on the device
    // (gbr_bundle_create, gbr_projector_upload per class,
    // gbr_model_set_arrays, gbr_bundle_set_optics); zeroed volumes sized
    // from image_current_size.  Replaces the previous iteration's bundle.
    void setupFixedSizedObjects();

    // Device-memory budget of the bundle and its workers (gbr_bundle_reserve).
    void setupTunableSizedObjects(size_t allocationSize);

    // The library's calls return after their work has completed.
    void syncAllBackprojects() {}

    // End of MlOptimiser::expectation: add the device volumes into
    // wsum_model.BPref and the weighted sums into wsum_model (as the
    // reference does after its threads, src/ml_optimiser.cpp:4380-4420).
    void storeWeightedSumsIntoModel();

    ~MlDeviceBundle();
};

class MlOptimiserCuda {
public:
    MlOptimiser *baseMLO;
    MlDeviceBundle *bundle;
    int device_id;
    bool refIs3D, dataIs3D;
    gbr_worker *worker = nullptr;

    MlOptimiserCuda(MlOptimiser *baseMLOptimiser, MlDeviceBundle *bundle, const char *timing_fnm);
    MlOptimiserCuda(const MlOptimiserCuda &) = delete;
    MlOptimiserCuda &operator=(const MlOptimiserCuda &) = delete;

    // Per-batch state lives in the library's worker: nothing to reset.
    void resetData() {}

    // The E-step of thread thread_id's share of the batch's particles
    // (contiguous, divide_equally over nr_threads): image preparation,
    // coarse and fine search, weights, weighted sums and backprojection in
    // one gbr_expect_images call; the results are written into the
    // particles' exp_metadata rows (ROT, TILT, PSI, XOFF, YOFF, CLASS, DLL,
    // PMAX, NR_SIGN, NORM).
    void doThreadExpectationSomeParticles(int thread_id);

    ~MlOptimiserCuda();
};

#endif
