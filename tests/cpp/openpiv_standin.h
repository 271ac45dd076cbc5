// openpiv_standin.h -- test-only container types with the interface of
// OpenPIV-c++'s core types (core/size.h, point.h, vector.h, rect.h,
// pixel_types.h, image.h, image_view.h) as far as the process example's
// per-window loop and openpiv_gpu.h use them.  The GPU machine has no
// reference sources, so the drop-in harness (process_dropin.cpp) is built
// there against these; on a machine with the reference it is also built
// against the reference's own headers.  Containers only: every algorithm the
// harness calls here (grid, correlation, peaks, fit) is openpiv::gpu's.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <ostream>
#include <stdexcept>
#include <vector>

namespace openpiv::algos {
enum class direction { FORWARD, REVERSE };
}

namespace openpiv::core {

class size {
public:
    size() = default;
    size(uint32_t w, uint32_t h) : w_(w), h_(h) {}
    uint32_t width() const { return w_; }
    uint32_t height() const { return h_; }
    uint32_t area() const { return w_ * h_; }
    bool operator==(const size& o) const { return w_ == o.w_ && h_ == o.h_; }
    bool operator!=(const size& o) const { return !(*this == o); }

private:
    uint32_t w_ = 0, h_ = 0;
};

inline std::ostream& operator<<(std::ostream& os, const size& s)
{
    return os << "[" << s.width() << "," << s.height() << "]";
}

// two components, indexable, convertible between component types
template <typename T>
class point2 {
public:
    using value_t = T;
    point2() = default;
    template <typename A, typename B>
    point2(A x, B y) : v_{ (T)x, (T)y } {}
    template <typename U>
    point2(const point2<U>& o) : v_{ (T)o[0], (T)o[1] } {}
    T& operator[](size_t i) { return v_[i]; }
    const T& operator[](size_t i) const { return v_[i]; }

private:
    std::array<T, 2> v_{};
};

template <typename T>
class vector2 {
public:
    vector2() = default;
    template <typename A, typename B>
    vector2(A x, B y) : v_{ (T)x, (T)y } {}
    T& operator[](size_t i) { return v_[i]; }
    const T& operator[](size_t i) const { return v_[i]; }

private:
    std::array<T, 2> v_{};
};

// bottom-left corner + size
class rect {
public:
    using point_t = point2<int32_t>;
    rect() = default;
    rect(const point_t& bl, const core::size& s) : bl_(bl), size_(s) {}
    static rect from_size(const core::size& s) { return rect({ 0, 0 }, s); }
    point_t bottomLeft() const { return bl_; }
    int32_t left() const { return bl_[0]; }
    int32_t bottom() const { return bl_[1]; }
    core::size size() const { return size_; }
    uint32_t width() const { return size_.width(); }
    uint32_t height() const { return size_.height(); }
    uint32_t area() const { return size_.area(); }
    // integer centre: bottom-left + size / 2
    point_t midpoint() const
    {
        return { bl_[0] + (int32_t)(size_.width() / 2), bl_[1] + (int32_t)(size_.height() / 2) };
    }
    // the centred rect of round(d * size), as the limited peak search uses
    rect dilate(double d) const
    {
        const int32_t w = (int32_t)width(), h = (int32_t)height();
        const int32_t rw = (int32_t)std::lround(d * w), rh = (int32_t)std::lround(d * h);
        return rect({ bl_[0] + (w - rw) / 2, bl_[1] + (h - rh) / 2 }, { (uint32_t)rw, (uint32_t)rh });
    }

private:
    point_t bl_{};
    core::size size_{};
};

// grey pixel: a value with implicit conversion both ways
template <typename T>
struct g {
    using value_t = T;
    g() = default;
    template <typename U>
    g(U x) : v((T)x) {}
    template <typename U>
    g& operator=(U x)
    {
        v = (T)x;
        return *this;
    }
    operator T() const { return v; }
    T v{};
};
using g_8 = g<uint8_t>;
using g_16 = g<uint16_t>;
using g_f = g<double>;

template <typename T>
struct complex {
    using value_t = T;
    complex() = default;
    template <typename U>
    complex(U r, U i = U{}) : real((T)r), imag((T)i) {}
    T real{}, imag{};
};
using c_f = complex<double>;

template <typename T>
class image {
public:
    using pixel_t = T;
    image() = default;
    image(uint32_t w, uint32_t h) : image(core::size{ w, h }) {}
    explicit image(const core::size& s) : r_(rect::from_size(s)), data_(s.area()) {}
    explicit image(const core::rect& r) : r_(r), data_(r.area()) {}
    uint32_t width() const { return r_.width(); }
    uint32_t height() const { return r_.height(); }
    core::size size() const { return r_.size(); }
    core::rect rect() const { return r_; }
    size_t pixel_count() const { return data_.size(); }
    T* line(size_t h) { return data_.data() + h * width(); }
    const T* line(size_t h) const { return data_.data() + h * width(); }
    T& operator[](const point2<uint32_t>& xy) { return line(xy[1])[xy[0]]; }
    const T& operator[](const point2<uint32_t>& xy) const { return line(xy[1])[xy[0]]; }

private:
    core::rect r_{};
    std::vector<T> data_;
};
using gf_image = image<g_f>;
using cf_image = image<c_f>;

// non-owning view of a rect of an image; rect() in the image's coordinates
// shifted by the image's own origin
template <typename T>
class image_view {
public:
    image_view() = default;
    image_view(const image<T>* im, const core::rect& r) : im_(im), r_(r) {}
    uint32_t width() const { return r_.width(); }
    uint32_t height() const { return r_.height(); }
    core::size size() const { return r_.size(); }
    core::rect rect() const
    {
        const core::rect ir = im_->rect();
        return core::rect({ ir.left() + r_.left(), ir.bottom() + r_.bottom() }, r_.size());
    }
    const T* line(size_t h) const { return im_->line(r_.bottom() + h) + r_.left(); }
    const T& operator[](const point2<uint32_t>& xy) const { return line(xy[1])[xy[0]]; }
    const image<T>& underlying() const { return *im_; }
    const core::rect& local() const { return r_; }

private:
    const image<T>* im_ = nullptr;
    core::rect r_{};
};

template <typename T>
using peaks_t = std::vector<image_view<T>>;

inline void check_inside(const core::rect& outer, const core::rect& r)
{
    if (r.left() < 0 || r.bottom() < 0 || (uint64_t)r.left() + r.width() > outer.width() ||
        (uint64_t)r.bottom() + r.height() > outer.height())
        throw std::out_of_range("image view not contained within image");
}

template <typename T>
image_view<T> create_image_view(const image<T>& im, core::rect r)
{
    check_inside(core::rect::from_size(im.size()), r);
    return image_view<T>(&im, r);
}

// a view of a view: r in the view's own coordinates
template <typename T>
image_view<T> create_image_view(const image_view<T>& v, core::rect r)
{
    check_inside(core::rect::from_size(v.size()), r);
    return image_view<T>(&v.underlying(),
                         core::rect({ v.local().left() + r.left(), v.local().bottom() + r.bottom() }, r.size()));
}

// a copy of a rect of an image that keeps the rect as its origin
template <typename T>
image<T> extract(const image<T>& im, core::rect r)
{
    check_inside(core::rect::from_size(im.size()), r);
    image<T> out(r);
    for (uint32_t h = 0; h < r.height(); ++h)
        for (uint32_t w = 0; w < r.width(); ++w) out.line(h)[w] = im.line(r.bottom() + h)[r.left() + w];
    return out;
}

}  // namespace openpiv::core
