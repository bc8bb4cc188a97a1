// Minimal stand-in for the few OpenCV core types the reference's walker sources name.
// It exists only so that the reference's CPU code can be compiled unmodified as a test
// oracle (see oracle/Makefile). Images never come from disk here: the oracle driver fills
// NMR_Simulation::binaryMap itself, so imread() always reports "no data".
#ifndef RWNMR_ORACLE_CV_CORE_SHIM_HPP
#define RWNMR_ORACLE_CV_CORE_SHIM_HPP

#include <cstddef>
#include <memory>
#include <string>
#include <vector>
#include <cassert>

typedef unsigned char uchar;

#define CV_8U 0
#define CV_8UC1 0
#define CV_Assert(expr) assert(expr)

namespace cv
{
using ::uchar;

// Single-channel 8-bit matrix with shared (reference-counted) storage, like cv::Mat.
class Mat
{
public:
    int rows = 0;
    int cols = 0;
    uchar *data = nullptr;

    Mat() {}
    Mat(int r, int c, int /*type*/) : rows(r), cols(c), store_(new std::vector<uchar>((size_t)r * (size_t)c, 0))
    {
        data = store_->data();
    }

    static Mat zeros(int r, int c, int type) { return Mat(r, c, type); }

    int channels() const { return 1; }
    int depth() const { return CV_8U; }

    template <typename T>
    T *ptr(int row) { return reinterpret_cast<T *>(data + (size_t)row * (size_t)cols); }
    template <typename T>
    const T *ptr(int row) const { return reinterpret_cast<const T *>(data + (size_t)row * (size_t)cols); }

private:
    std::shared_ptr<std::vector<uchar>> store_;
};

inline Mat imread(const std::string &, int = 0) { return Mat(); }
} // namespace cv

#endif
