// Test infrastructure: the part of the Blitz++ Array interface that the reference's CPU
// services use (src/services/{count,countLeft,partition,makeAxis}.cpp and pst.h), written
// here so those files compile unchanged without Blitz++ (which the image does not have).
// Arrays are views over memory the test driver owns: element (i, j) of a 2-D array sits at
// data[i * stride0 + j * stride1]; copying an array copies the view (Blitz++'s reference
// semantics); a Range is inclusive of both ends (Blitz++'s convention).
#ifndef ORB_REFSHIM_BLITZ_ARRAY_H
#define ORB_REFSHIM_BLITZ_ARRAY_H

#include <cstddef>

namespace blitz {

struct Range {
    int first_, last_;
    Range(int first, int last) : first_(first), last_(last) {}
};

template <int N>
struct ColumnMajorArray {};

template <class T, int N>
class Array;

template <class T>
class Array<T, 1> {
   public:
    Array() : p_(nullptr), n_(0), s_(1) {}
    Array(T *p, int n, std::ptrdiff_t stride = 1) : p_(p), n_(n), s_(stride) {}
    T &operator()(int i) const { return p_[i * s_]; }
    Array operator()(Range r) const { return Array(p_ + r.first_ * s_, r.last_ - r.first_ + 1, s_); }
    T *data() const { return p_; }
    int rows() const { return n_; }
    int extent(int) const { return n_; }

   private:
    T *p_;
    int n_;
    std::ptrdiff_t s_;
};

template <class T>
class Array<T, 2> {
   public:
    Array() : p_(nullptr), r_(0), c_(0), s0_(0), s1_(0) {}
    Array(T *p, int rows, int cols, std::ptrdiff_t s0, std::ptrdiff_t s1)
        : p_(p), r_(rows), c_(cols), s0_(s0), s1_(s1) {}
    T &operator()(int i, int j) const { return p_[i * s0_ + j * s1_]; }
    // a column segment: rows [first, last] of column j
    Array<T, 1> operator()(Range r, int j) const {
        return Array<T, 1>(p_ + r.first_ * s0_ + j * s1_, r.last_ - r.first_ + 1, s0_);
    }
    T *data() const { return p_; }
    int rows() const { return r_; }
    int columns() const { return c_; }

   private:
    T *p_;
    int r_, c_;
    std::ptrdiff_t s0_, s1_;
};

}  // namespace blitz

#endif
