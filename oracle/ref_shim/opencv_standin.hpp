// TEST INFRASTRUCTURE ONLY -- stand-in for the parts of OpenCV's cv::Mat that
// the reference's CPU DIC sources use: an 8-bit single-channel image with
// rows, cols and at<uchar>(row, col).  Copies share the pixel buffer, as
// cv::Mat's reference-counted copies do; the caller keeps the buffer alive.
// The reference includes OpenCV with Windows path separators
// (opencv2\opencv.hpp and others); oracle/build_ref.py writes forwarding
// headers of those literal names that include this file.
#ifndef TWREF_OPENCV_STANDIN_HPP
#define TWREF_OPENCV_STANDIN_HPP

#include <cstddef>
#include <cstdint>

typedef unsigned char uchar;

#define CV_8UC1 0

namespace cv {

class Mat {
public:
    int rows = 0;
    int cols = 0;
    uchar* data = nullptr;
    size_t step = 0;

    Mat() = default;
    Mat(int rows_, int cols_, int /*type*/, void* data_, size_t step_ = 0)
        : rows(rows_), cols(cols_), data(static_cast<uchar*>(data_)), step(step_ ? step_ : (size_t)cols_) {}

    template <typename T>
    T& at(int r, int c) { return reinterpret_cast<T*>(data + (size_t)r * step)[c]; }
    template <typename T>
    const T& at(int r, int c) const { return reinterpret_cast<const T*>(data + (size_t)r * step)[c]; }
    bool empty() const { return data == nullptr; }
};

}  // namespace cv

#endif
