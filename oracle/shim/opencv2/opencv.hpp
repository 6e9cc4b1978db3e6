// Stand-in for the OpenCV subset the reference segmenter uses (8-bit images, split/merge,
// 5x5 rectangular dilation, no-op display calls). Test infrastructure only.
//
// cv::dilate is restated from OpenCV's documented behaviour: the output pixel is the maximum
// over the structuring element's window centred on the pixel; with the default border
// (BORDER_CONSTANT + morphologyDefaultBorderValue) pixels outside the image never win, i.e.
// the window is clipped to the image and there is no wrap-around.
#pragma once
#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

namespace cv
{
typedef unsigned char uchar;

enum
{
    CV_8U = 0
};
#define CV_8UC1 0
#define CV_8UC3 16

enum
{
    MORPH_RECT = 0
};

struct Size
{
    int width;
    int height;
    Size(int w, int h) : width(w), height(h) {}
};

struct Scalar
{
    double v[4];
    Scalar(double a = 0, double b = 0, double c = 0, double d = 0) : v{a, b, c, d} {}
};

struct Vec3b
{
    uchar val[3];
    Vec3b() : val{0, 0, 0} {}
    Vec3b(uchar a, uchar b, uchar c) : val{a, b, c} {}
    uchar& operator[](int i) { return val[i]; }
    const uchar& operator[](int i) const { return val[i]; }
    bool operator==(const Vec3b& o) const
    {
        return val[0] == o.val[0] && val[1] == o.val[1] && val[2] == o.val[2];
    }
    bool operator!=(const Vec3b& o) const { return !(*this == o); }
};

class Mat
{
  public:
    int rows{0};
    int cols{0};
    int channels_{1};
    std::vector<uchar> buf;

    Mat() = default;
    Mat(int r, int c, int type) { create(r, c, type); }

    static Mat zeros(int r, int c, int type) { return Mat(r, c, type); }

    void create(int r, int c, int type)
    {
        rows = r;
        cols = c;
        channels_ = (type == CV_8UC3) ? 3 : 1;
        buf.assign(static_cast<std::size_t>(r) * c * channels_, 0);
    }

    int depth() const { return CV_8U; }
    int channels() const { return channels_; }

    void setTo(const Scalar& s)
    {
        for (std::size_t i = 0; i < buf.size(); ++i)
        {
            buf[i] = static_cast<uchar>(s.v[i % channels_]);
        }
    }

    template <typename T>
    T& at(int r, int c);
    template <typename T>
    const T& at(int r, int c) const;
};

template <>
inline Vec3b& Mat::at<Vec3b>(int r, int c)
{
    return *reinterpret_cast<Vec3b*>(&buf[(static_cast<std::size_t>(r) * cols + c) * 3]);
}
template <>
inline const Vec3b& Mat::at<Vec3b>(int r, int c) const
{
    return *reinterpret_cast<const Vec3b*>(&buf[(static_cast<std::size_t>(r) * cols + c) * 3]);
}
template <>
inline uchar& Mat::at<uchar>(int r, int c)
{
    return buf[static_cast<std::size_t>(r) * cols + c];
}
template <>
inline const uchar& Mat::at<uchar>(int r, int c) const
{
    return buf[static_cast<std::size_t>(r) * cols + c];
}

inline Mat getStructuringElement(int /*shape*/, Size ksize)
{
    Mat k(ksize.height, ksize.width, CV_8UC1);
    std::fill(k.buf.begin(), k.buf.end(), 1);
    return k;
}

inline void split(const Mat& src, std::vector<Mat>& dst)
{
    dst.resize(src.channels_);
    for (int ch = 0; ch < src.channels_; ++ch)
    {
        dst[ch].create(src.rows, src.cols, CV_8UC1);
        for (std::size_t i = 0; i < static_cast<std::size_t>(src.rows) * src.cols; ++i)
        {
            dst[ch].buf[i] = src.buf[i * src.channels_ + ch];
        }
    }
}

inline void merge(const std::vector<Mat>& src, Mat& dst)
{
    const int nch = static_cast<int>(src.size());
    dst.create(src[0].rows, src[0].cols, nch == 3 ? CV_8UC3 : CV_8UC1);
    for (int ch = 0; ch < nch; ++ch)
    {
        for (std::size_t i = 0; i < static_cast<std::size_t>(dst.rows) * dst.cols; ++i)
        {
            dst.buf[i * nch + ch] = src[ch].buf[i];
        }
    }
}

// Rectangular dilation with an all-ones kernel anchored at its centre, window clipped to the
// image (the default constant border never wins a max).
inline void dilate(const Mat& src, Mat& dst, const Mat& kernel)
{
    const int kh = kernel.rows;
    const int kw = kernel.cols;
    const int ah = kh / 2;
    const int aw = kw / 2;
    Mat out(src.rows, src.cols, CV_8UC1);
    for (int r = 0; r < src.rows; ++r)
    {
        for (int c = 0; c < src.cols; ++c)
        {
            uchar m = 0;
            for (int dr = -ah; dr < kh - ah; ++dr)
            {
                const int rr = r + dr;
                if (rr < 0 || rr >= src.rows)
                {
                    continue;
                }
                for (int dc = -aw; dc < kw - aw; ++dc)
                {
                    const int cc = c + dc;
                    if (cc < 0 || cc >= src.cols)
                    {
                        continue;
                    }
                    m = std::max(m, src.buf[static_cast<std::size_t>(rr) * src.cols + cc]);
                }
            }
            out.buf[static_cast<std::size_t>(r) * src.cols + c] = m;
        }
    }
    dst = out;
}

inline void flip(const Mat& src, Mat& dst, int /*code*/) { dst = src; }
inline void imshow(const std::string&, const Mat&) {}
inline int waitKey(int) { return -1; }
} // namespace cv
