// ref_multicore.cpp -- host build of the reference's Kinect pre-processing
// routines (test infrastructure, built only by oracle/build_ref.py into
// oracle/_ref/libreconref.so).  OMPFunctions' d2Z, d2ZLow, convert2Gray,
// undistort and undistortLookup are extracted verbatim from
// tracker/multicore/multicore.cpp into oracle/_ref/frag_multicore.inc; this
// file supplies the little of OpenCV's Mat and of the OMPFunctions class they
// use, and exports ref_* wrappers.
#include <assert.h>
#include <math.h>
#include <string.h>

#include <vector>

// the members of cv::Mat the routines use
struct Mat {
    int rows = 0, cols = 0;
    unsigned char *data = nullptr;
    unsigned char *ptr() { return data; }
};

class OMPFunctions {
public:
    int NTHR = 64;
    bool mappingPrecomputed = false;
    float *dxTable = nullptr;
    void d2Z(Mat &dispImage, Mat &depthImage, float c0, float c1, float minDist, float maxDist, float xOff, float yOff);
    void d2ZLow(Mat &dispImage, Mat &depthImageSmall, float c0, float c1, float minDist, float maxDist, float xOff,
                float yOff);
    void convert2Gray(Mat &rgbImage, Mat &grayImage);
    void undistort(Mat &src, Mat &dst, float *K, float *iK, float *kc);
    void undistortLookup(Mat &src, Mat &dst);
};

#include "frag_multicore.inc"

static Mat mat(void *p, int rows, int cols) {
    Mat m;
    m.rows = rows;
    m.cols = cols;
    m.data = (unsigned char *)p;
    return m;
}

extern "C" {

void ref_d2Z(unsigned short *disp, int W, int H, float c0, float c1, float mind, float maxd, float xo, float yo,
             float *z) {
    OMPFunctions f;
    Mat d = mat(disp, H, W), zz = mat(z, H, W);
    f.d2Z(d, zz, c0, c1, mind, maxd, xo, yo);
}

void ref_d2ZLow(unsigned short *disp, int Wl, int Hl, float c0, float c1, float mind, float maxd, float xo, float yo,
                float *z) {
    OMPFunctions f;
    Mat d = mat(disp, 2 * Hl, 2 * Wl), zz = mat(z, Hl, Wl);
    f.d2ZLow(d, zz, c0, c1, mind, maxd, xo, yo);
}

void ref_convert2Gray(unsigned char *rgb, int W, int H, unsigned char *gray) {
    OMPFunctions f;
    Mat a = mat(rgb, H, W), b = mat(gray, H, W);
    f.convert2Gray(a, b);
}

// `calls` calls of undistort on copies of src (the first computes the mapping,
// later ones use undistortLookup); dst receives the last result
void ref_undistort(unsigned char *src, int W, int H, float *K, float *iK, float *kc, int calls, unsigned char *dst) {
    OMPFunctions f;
    std::vector<float> table(2 * (size_t)W * H);
    f.dxTable = table.data();
    std::vector<unsigned char> s(src, src + (size_t)W * H);
    for (int i = 0; i < calls; i++) {
        memcpy(s.data(), src, s.size());
        Mat a = mat(s.data(), H, W), b = mat(dst, H, W);
        f.undistort(a, b, K, iK, kc);
    }
}

}  // extern "C"
