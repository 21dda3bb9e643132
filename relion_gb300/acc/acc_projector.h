// acc_projector.h -- AccProjector of the GB300 façade.
//
// The reference's AccProjector (src/acc/acc_projector.h:17-104) owns the
// device copy of one class's padded Fourier reference (texture objects or a
// complex array).  Here the copy lives in a libgbrelion bundle at one class
// index: setMdlDim records the geometry, initMdl uploads the data
// (gbr_projector_upload), and the bundle frees it.
#ifndef GB300_ACC_PROJECTOR_H
#define GB300_ACC_PROJECTOR_H

#include <vector>

#include "gbrelion.h"
#include "ml_optimiser_stub.h"

typedef float XFLOAT;

class AccProjector {
    int mdlX = 0, mdlY = 0, mdlZ = 0, mdlMaxR = 0, mdlInitY = 0, mdlInitZ = 0;
    XFLOAT padding_factor = 0;
    size_t mdlXYZ = 0;
    gbr_bundle *bundle = nullptr;
    long iclass = -1;

public:
    AccProjector() = default;

    // the bundle and class this projector fills (set by MlDeviceBundle)
    void attach(gbr_bundle *b, long cls) {
        bundle = b;
        iclass = cls;
    }

    // Geometry of the model; true when it differs from the previous one
    // (the reference then reallocates its device arrays).
    bool setMdlDim(int xdim, int ydim, int zdim, int inity, int initz, int maxr, XFLOAT paddingFactor);

    // Upload the model (split or complex form, as the reference's two
    // variants); throws std::runtime_error with the library's message.
    void initMdl(const XFLOAT *real, const XFLOAT *imag);
    void initMdl(const Complex *data);

    void clear();
    ~AccProjector() { clear(); }
};

#endif
