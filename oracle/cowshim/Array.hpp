// Clean-room stand-in for the container types Mara2 takes from its Cow
// submodule (jzrake/Cow2), which is not vendored with the reference.  It is
// written from the behaviour described in the reference's manual
// (Doc/Manual/manual.tex, "Review on Cow") and exercised by its container
// tests (src/TestSuite.cpp:14-345), and implements only what the hot-path
// translation units use.  TEST INFRASTRUCTURE: it exists so the oracle can
// compile the reference's own sources; nothing in the product links it.
//
// Conventions:
//   * Shape / Index are 5-vectors; arrays are 5-D, C order (axis 4 fastest).
//   * Region lower/upper/stride per axis; a lower < 0 or an upper <= 0 counts
//     from the end of the axis (upper 0 == the axis length).
//   * Iterators walk a region in C order; two iterators compare by the
//     element address, and every exhausted iterator over the same array and
//     axis-0 range points one past the region on axis 0, so a strided walk
//     ends where an unstrided walk of the same region ends.
#pragma once

#include <array>
#include <cstring>
#include <functional>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace Cow
{
using Shape = std::array<int, 5>;
using Index = std::array<int, 5>;

class Array;

// ============================================================================
class Shape3D
{
public:
    Shape3D() : S {{0, 0, 0, 1, 1}} {}
    Shape3D (int n0, int n1, int n2) : S {{n0, n1, n2, 1, 1}} {}
    Shape3D (Shape shape) : S (shape) {}
    Shape3D (const Array& A);

    int& operator[] (int axis) { return S[axis]; }
    const int& operator[] (int axis) const { return S[axis]; }
    operator Shape() const { return S; }

    Shape3D increased (int delta = 1) const { auto R = *this; for (int a = 0; a < 3; ++a) R.S[a] += delta; return R; }
    Shape3D increased (int axis, int delta) const { auto R = *this; R.S[axis] += delta; return R; }
    Shape3D increased (const Shape3D& d) const { auto R = *this; for (int a = 0; a < 3; ++a) R.S[a] += d.S[a]; return R; }
    Shape3D reduced (int delta) const { return increased (-delta); }
    Shape3D reduced (int axis, int delta) const { return increased (axis, -delta); }
    Shape3D withComponents (int n) const { auto R = *this; R.S[3] = n; return R; }
    Shape3D withRank (int n) const { auto R = *this; R.S[4] = n; return R; }

    bool contains (const Shape3D& other) const
    {
        for (int a = 0; a < 3; ++a) if (S[a] < other.S[a]) return false;
        return true;
    }
    Shape3D operator* (int f) const { auto R = *this; for (int a = 0; a < 3; ++a) R.S[a] *= f; return R; }
    Shape3D operator/ (int f) const { auto R = *this; for (int a = 0; a < 3; ++a) R.S[a] /= f; return R; }

    void deploy (std::function<void (int, int, int)> f) const
    {
        for (int i = 0; i < S[0]; ++i)
            for (int j = 0; j < S[1]; ++j)
                for (int k = 0; k < S[2]; ++k)
                    f (i, j, k);
    }

private:
    Shape S;
};

// ============================================================================
struct Region
{
    Region() : lower {{0, 0, 0, 0, 0}}, upper {{0, 0, 0, 0, 0}}, stride {{1, 1, 1, 1, 1}} {}
    Region (Shape shape) : Region() { upper = shape; }

    Region withRange (int axis, int lo, int hi, int st = 1) const
    {
        auto R = *this; R.lower[axis] = lo; R.upper[axis] = hi; R.stride[axis] = st; return R;
    }
    Region withStride (int axis, int st) const { auto R = *this; R.stride[axis] = st; return R; }
    Region withLower (int axis, int lo) const { auto R = *this; R.lower[axis] = lo; return R; }
    Region withUpper (int axis, int hi) const { auto R = *this; R.upper[axis] = hi; return R; }

    /** Resolve end-relative bounds against an array shape. */
    Region absolute (Shape arrayShape) const
    {
        auto R = *this;
        for (int a = 0; a < 5; ++a)
        {
            if (R.lower[a] < 0) R.lower[a] += arrayShape[a];
            if (R.upper[a] <= 0) R.upper[a] += arrayShape[a];
        }
        return R;
    }
    /** Number of visited points per axis (bounds must be absolute). */
    Shape shape() const
    {
        Shape s;
        for (int a = 0; a < 5; ++a)
        {
            const int n = upper[a] - lower[a];
            s[a] = n <= 0 ? 0 : (n + stride[a] - 1) / stride[a];
        }
        return s;
    }

    Index lower;
    Index upper;
    Index stride;
};

// ============================================================================
class Array
{
public:
    class Reference;

    class Iterator
    {
    public:
        Iterator (double* base, Shape arrayShape, Region absRegion, bool atEnd) :
        base (base), N (arrayShape), R (absRegion)
        {
            idx = R.lower;
            if (atEnd || empty()) idx[0] = R.upper[0];
            ptr = base + offset (idx);
        }
        Iterator& operator++()
        {
            for (int a = 4; a >= 0; --a)
            {
                idx[a] += R.stride[a];
                if (a == 0 && idx[0] >= R.upper[0]) { idx[0] = R.upper[0]; break; }
                if (idx[a] < R.upper[a]) break;
                idx[a] = R.lower[a];
            }
            ptr = base + offset (idx);
            return *this;
        }
        bool operator== (const Iterator& other) const { return ptr == other.ptr; }
        bool operator!= (const Iterator& other) const { return ptr != other.ptr; }
        double& operator*() const { return *ptr; }
        double& operator[] (int n) const { return ptr[n]; }
        operator double*() const { return ptr; }
        Index index() const { return idx; }
        Index relativeIndex() const { Index r; for (int a = 0; a < 5; ++a) r[a] = idx[a] - R.lower[a]; return r; }

    private:
        bool empty() const { for (int a = 0; a < 5; ++a) if (R.upper[a] <= R.lower[a]) return true; return false; }
        long offset (const Index& I) const
        {
            long o = 0;
            for (int a = 0; a < 5; ++a) o = o * N[a] + I[a];
            return o;
        }
        double* base;
        Shape N;
        Region R;
        Index idx;
        double* ptr;
    };

    class Reference
    {
    public:
        Reference (Array& A, Region R) : A (&A), R (R) {}
        Reference (Array& A) : A (&A), R() {}
        Reference (const Reference& other) = default;

        Reference& operator= (const Array& source) { assign (source.data(), source.shape(), Region()); return *this; }
        Reference& operator= (const Reference& source)
        {
            assign (source.A->data(), source.A->shape(), source.R);
            return *this;
        }
        Array& getArray() const { return *A; }
        Region getRegion() const { return R; }
        Shape shape() const { return R.absolute (A->shape()).shape(); }
        int size (int axis) const { return shape()[axis]; }
        int size() const { auto s = shape(); return s[0] * s[1] * s[2] * s[3] * s[4]; }
        Iterator begin() const { return Iterator (A->data(), A->shape(), R.absolute (A->shape()), false); }
        Iterator end() const { return Iterator (A->data(), A->shape(), R.absolute (A->shape()), true); }

    private:
        void assign (const double* src, Shape srcShape, Region srcRegion)
        {
            // Copy element-wise: both regions are walked in C order.
            const Region sr = srcRegion.absolute (srcShape);
            if (sr.shape() != shape())
                throw std::logic_error ("Cow shim: assignment between regions of different shape");
            std::vector<double> tmp;
            for (auto it = Iterator (const_cast<double*> (src), srcShape, sr, false),
                 e = Iterator (const_cast<double*> (src), srcShape, sr, true); it != e; ++it)
                tmp.push_back (*it);
            std::size_t n = 0;
            for (auto it = begin(); it != end(); ++it) *it = tmp[n++];
        }
        Array* A;
        Region R;
    };

    Array() : S {{0, 1, 1, 1, 1}} {}
    explicit Array (int n0, int n1 = 1, int n2 = 1, int n3 = 1, int n4 = 1) : S {{n0, n1, n2, n3, n4}}, D (count (S), 0.0) {}
    Array (Shape shape) : S (shape), D (count (S), 0.0) {}
    Array (Shape3D shape) : Array (Shape (shape)) {}
    Array (const Reference& ref) : S (ref.shape()), D()
    {
        D.reserve (count (S));
        for (auto it = ref.begin(); it != ref.end(); ++it) D.push_back (*it);
    }
    Array (const Array&) = default;
    Array& operator= (const Array&) = default;
    Array (Array&& other) noexcept : S (other.S), D (std::move (other.D)) { other.S = Shape {{0, 1, 1, 1, 1}}; other.D.clear(); }
    Array& operator= (Array&& other) noexcept
    {
        if (this != &other) { S = other.S; D = std::move (other.D); other.S = Shape {{0, 1, 1, 1, 1}}; other.D.clear(); }
        return *this;
    }

    double& operator() (int i, int j = 0, int k = 0, int q = 0, int r = 0) { return D[at (i, j, k, q, r)]; }
    const double& operator() (int i, int j = 0, int k = 0, int q = 0, int r = 0) const { return D[at (i, j, k, q, r)]; }
    double& operator[] (int n) { return D[n]; }
    const double& operator[] (int n) const { return D[n]; }
    Reference operator[] (Region R) { return Reference (*this, R); }

    int size() const { return int (D.size()); }
    int size (int axis) const { return S[axis]; }
    Shape shape() const { return S; }
    Shape3D shape3D() const { return Shape3D (S); }
    double* data() { return D.data(); }
    const double* data() const { return D.data(); }

    /** Copy the elements of `source` (a region of src) into the region
        `target` of this array; both are walked in C order and must have the
        same extents. */
    void copyFrom (const Array& src, Region target, Region source)
    {
        Reference (*this, target) = Reference (const_cast<Array&> (src), source);
    }

    Iterator begin() { return Iterator (data(), S, Region().absolute (S), false); }
    Iterator end() { return Iterator (data(), S, Region().absolute (S), true); }

    static void deploy (Shape3D shape, std::function<void (int, int, int)> f) { shape.deploy (f); }
    static bool isBoundsCheckDisabled() { return true; }

private:
    static std::size_t count (const Shape& s) { long n = 1; for (int a = 0; a < 5; ++a) n *= s[a]; return n < 0 ? 0 : std::size_t (n); }
    long at (int i, int j, int k, int q, int r) const
    {
        return ((((long) i * S[1] + j) * S[2] + k) * S[3] + q) * S[4] + r;
    }
    Shape S;
    std::vector<double> D;
};

inline Shape3D::Shape3D (const Array& A) : S (A.shape()) {}

} // namespace Cow
