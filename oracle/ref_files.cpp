// ref_files.cpp -- host wrappers of the reference's result-file classes (test
// infrastructure, built only by oracle/build_ref.py into
// oracle/_ref/libreconref.so): ResultTxt (tracker/calib/ResultTxt.cpp) and
// TrackingParams (tracker/calib/TrackingParams.cpp), compiled from the
// reference's own sources.
#include "calib/ResultTxt.h"
#include "calib/TrackingParams.h"

extern "C" {

// ResultTxt::init(fn, add_identity), addPose for every pose, save(transpose, inverse)
void ref_result_save(const char *fn, float *poses, int n, int add_identity, int transpose, int inverse) {
    ResultTxt r;
    r.init(fn, add_identity != 0);
    for (int i = 0; i < n; i++) r.addPose(&poses[16 * i]);
    r.save(transpose, inverse);
}

// TrackingParams::init(fn) and getParams(frame_key)
void ref_track_params_get(const char *fn, int frame_key, int *frame, int *mode, float *lambda) {
    TrackingParams p;
    p.init(fn);
    TRACK_PARAMS *t = p.getParams(frame_key);
    *frame = t->frame;
    *mode = (int)t->trackMode;
    *lambda = t->lambda;
}

}  // extern "C"
