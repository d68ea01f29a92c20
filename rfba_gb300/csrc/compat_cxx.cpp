// C++-linkage aliases of the reference exports.
//
// RFBA Main/GradientCalc/GradientCalc.h:4-5 declares SRRFGradientCalc and
// SRRFGetMag without extern "C", so a caller compiled against that header
// (multispot5_place_methods.cc:48-49, multispot5.cc:77) binds the C++-mangled
// symbols. This file exports those mangled names and forwards them to the
// extern "C" entry points of include/rfba_srrf.h, so both kinds of caller link
// against librfba_srrf.so unchanged. (SRRFGradientCalcGPU is extern "C" in the
// reference, kernel.cuh:26, and needs no alias.)
extern "C" int rfba_compat_gradientcalc(float* in, int* dims, float* out);
extern "C" int rfba_compat_getmag(void);

int SRRFGradientCalc(float* inImage, int* imageDim, float* outImage) {
    return rfba_compat_gradientcalc(inImage, imageDim, outImage);
}

int SRRFGetMag() { return rfba_compat_getmag(); }
