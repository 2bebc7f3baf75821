/*
 * opencv2/opencv.hpp -- compile-only stub of the few OpenCV names the
 * reference's olimg.h mentions (cv::Mat, imread, imwrite, flip, cvtColor;
 * olimg.h:105-175).  TEST INFRASTRUCTURE ONLY: OpenCV is not installed here and
 * image file IO is outside the propagation/CGH path, so these bodies only
 * return empty images; nothing in the oracle calls them.
 */
#ifndef OL_OPENCV_STUB_HPP
#define OL_OPENCV_STUB_HPP
#include <cstdint>
#include <cstring>
#include <string>
#include <sstream>
#include <stdexcept>

#define CV_8U 0
namespace cv {
enum { COLOR_BGR2GRAY = 6 };
struct Mat {
    int rows = 0, cols = 0, type_ = 0;
    unsigned char *data = nullptr;
    Mat() {}
    Mat(int r, int c, int t, void *d) : rows(r), cols(c), type_(t), data((unsigned char *)d) {}
    template <typename T> T &at(int r, int c) { return ((T *)data)[r * cols + c]; }
    void release() { data = nullptr; rows = cols = 0; }
};
inline Mat imread(const std::string &) { throw std::runtime_error("opencv stub: imread unavailable"); }
inline bool imwrite(const std::string &, const Mat &) { throw std::runtime_error("opencv stub: imwrite unavailable"); }
inline void flip(const Mat &, Mat &, int) {}
inline void cvtColor(const Mat &, Mat &, int) {}
} // namespace cv
#endif
