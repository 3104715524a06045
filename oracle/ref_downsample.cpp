// ref_downsample.cpp -- C entry points over the reference's host pyramid
// construction (src/PaintTweenCUDA/downsample.cpp), compiled with it from
// the reference tree, over the QtCore container shim in oracle/qt_shim, into
// oracle/_ref/libref_helpers.so by oracle/build.py.
//
// Test infrastructure only.  Each entry point builds the whole pyramid of a
// w x h image and writes its levels one after another into `out` (level 0,
// the input itself, first); it returns the number of levels.  `out` must
// hold sum over levels of (w >> l) * (h >> l) elements of the pixel type.
#include <cstring>

#include "downsample.h"

namespace {

template <class T>
int pyramid(const T* in, int w, int h, int mode, T* out) {
    QVector<T> input(w * h);
    std::memcpy(input.data(), in, sizeof(T) * (size_t)w * (size_t)h);
    QList<QVector<T> > levels;
    downsamplePyramid<T>(input, levels, w, h, mode ? DOWNSAMPLE_SCALE_WITH_LEVELS : DOWNSAMPLE_SCALE_CONSTANT);
    size_t off = 0;
    for (int l = 0; l < levels.size(); ++l) {
        size_t n = (size_t)levels[l].size();
        std::memcpy(out + off, levels[l].constData(), sizeof(T) * n);
        off += n;
    }
    return levels.size();
}

}  // namespace

extern "C" {

int ref_pyramid_rgba(const float* in, int w, int h, int mode, float* out) {
    return pyramid<Color4>(reinterpret_cast<const Color4*>(in), w, h, mode, reinterpret_cast<Color4*>(out));
}
int ref_pyramid_float(const float* in, int w, int h, int mode, float* out) {
    return pyramid<float>(in, w, h, mode, out);
}
int ref_pyramid_float2(const float* in, int w, int h, int mode, float* out) {
    return pyramid<float2>(reinterpret_cast<const float2*>(in), w, h, mode, reinterpret_cast<float2*>(out));
}
int ref_pyramid_int(const int* in, int w, int h, int* out) { return pyramid<int>(in, w, h, 0, out); }

}  // extern "C"
