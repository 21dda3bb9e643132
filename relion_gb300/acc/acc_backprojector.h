// acc_backprojector.h -- AccBackprojector of the GB300 façade.
//
// The reference's AccBackprojector (src/acc/acc_backprojector.h:24-99) holds
// one class's device volumes (real, imaginary, weight) into which
// storeWeightedSums backprojects each particle's weighted images.  Here the
// volumes (FP64) live in a libgbrelion bundle: the batch call
// (gbr_expect_batch / gbr_expect_images) backprojects into them itself, so
// there is no separate backproject() launch; getMdlData reads them back
// (gbr_backprojector_download).
#ifndef GB300_ACC_BACKPROJECTOR_H
#define GB300_ACC_BACKPROJECTOR_H

#include <vector>

#include "acc_projector.h"

class AccBackprojector {
public:
    int mdlX = 0, mdlY = 0, mdlZ = 0, mdlInitY = 0, mdlInitZ = 0, maxR = 0, maxR2 = 0;
    XFLOAT padding_factor = 0;
    size_t mdlXYZ = 0;

    AccBackprojector() = default;

    void attach(gbr_bundle *b, long cls) {
        bundle = b;
        iclass = cls;
    }

    // Geometry of the volumes; returns the number of voxels.  The bundle
    // sizes its volumes from current_size: a geometry that differs from the
    // bundle's is rejected (std::runtime_error).
    size_t setMdlDim(int xdim, int ydim, int zdim, int inity, int initz, int max_r, XFLOAT paddingFactor);

    // Zero the volumes (with the bundle's weighted sums: gbr_bundle_reset_wsum).
    void initMdl();

    // Read back the accumulated volumes, [z][y][x].  The FP64 form is exact;
    // the XFLOAT form is the reference's signature (rounded to float).
    void getMdlData(double *real, double *imag, double *weights);
    void getMdlData(XFLOAT *real, XFLOAT *imag, XFLOAT *weights);

    void clear();
    ~AccBackprojector() { clear(); }

private:
    gbr_bundle *bundle = nullptr;
    long iclass = -1;
};

#endif
