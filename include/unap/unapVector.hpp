/* UNAP::Vector<T>: the reference's host vector (src/base/vectors/
 * unapVector.hpp), with scalarField = Vector<scalar> and labelField =
 * Vector<label>.  A vector built on borrowed memory (reUse) does not free
 * it. */
#ifndef UNAPVECTOR_HPP
#define UNAPVECTOR_HPP

#include "unap.hpp"

namespace UNAP
{

template <typename T>
class Vector
{
private:
    label length_;
    T* values_;
    bool owns_;

    void alloc(label n)
    {
        length_ = n;
        values_ = n > 0 ? new T[n] : NULL;
        owns_ = true;
    }

public:
    Vector() : length_(0), values_(NULL), owns_(true) {}

    explicit Vector(const label length)
    {
        alloc(length);
        forAll(i, length_) values_[i] = T(0);
    }

    Vector(const Vector<T>& v)
    {
        alloc(v.length_);
        forAll(i, length_) values_[i] = v.values_[i];
    }

    Vector(const T* val, const label& length)
    {
        alloc(length);
        forAll(i, length_) values_[i] = val[i];
    }

    Vector(const T* val, const label& length, const bool reUse)
    {
        if (reUse) {
            length_ = length;
            values_ = const_cast<T*>(val);
            owns_ = false;
        } else {
            alloc(length);
            forAll(i, length_) values_[i] = val[i];
        }
    }

    Vector(const label len, const T value)
    {
        alloc(len);
        forAll(i, length_) values_[i] = value;
    }

    virtual ~Vector()
    {
        if (owns_) delete[] values_;
        values_ = NULL;
    }

    inline T& operator[](const label i) { return values_[i]; }
    inline const T operator[](const label i) const { return values_[i]; }

    Vector& operator=(const Vector<T>& v)
    {
        if (&v == this) return *this;
        if (length_ != v.length_) {
            if (owns_) delete[] values_;
            alloc(v.length_);
        }
        forAll(i, length_) values_[i] = v.values_[i];
        return *this;
    }

    Vector& operator=(const T& a)
    {
        forAll(i, length_) values_[i] = a;
        return *this;
    }

    Vector& operator+=(const Vector<T>& v)
    {
        forAll(i, length_) values_[i] += v.values_[i];
        return *this;
    }
    Vector& operator-=(const Vector<T>& v)
    {
        forAll(i, length_) values_[i] -= v.values_[i];
        return *this;
    }
    Vector& operator+=(const T& a)
    {
        forAll(i, length_) values_[i] += a;
        return *this;
    }
    Vector& operator-=(const T& a)
    {
        forAll(i, length_) values_[i] -= a;
        return *this;
    }
    Vector& operator*=(const T& a)
    {
        forAll(i, length_) values_[i] *= a;
        return *this;
    }

    const Vector operator+(const Vector<T>& v) const
    {
        Vector r(*this);
        r += v;
        return r;
    }
    const Vector operator-(const Vector<T>& v) const
    {
        Vector r(*this);
        r -= v;
        return r;
    }
    const Vector operator*(const T& a) const
    {
        Vector r(*this);
        r *= a;
        return r;
    }

    label size() const { return length_; }

    /* resize, keeping the first min(old, new) values */
    void SET_size(const label newSize)
    {
        if (newSize == length_) return;
        T* nv = newSize > 0 ? new T[newSize] : NULL;
        const label keep = MIN(length_, newSize);
        for (label i = 0; i < keep; ++i) nv[i] = values_[i];
        if (owns_) delete[] values_;
        values_ = nv;
        length_ = newSize;
        owns_ = true;
    }

    T* values() const { return values_; }
    T* begin() const { return values_; }

    void SET_zero()
    {
        forAll(i, length_) values_[i] = T(0);
    }

    /* sums over this process's entries (one rank: no reduction) */
    T Sum() const
    {
        T s = 0;
        forAll(i, length_) s += values_[i];
        return s;
    }
    T SumMag() const
    {
        T s = 0;
        forAll(i, length_) s += mag(values_[i]);
        return s;
    }
    T SumSqr() const
    {
        T s = 0;
        forAll(i, length_) s += values_[i] * values_[i];
        return s;
    }
    scalar SumSqrt() const { return sqrt((scalar)SumSqr()); }
};

typedef Vector<scalar> scalarField;
typedef Vector<label> labelField;

inline scalar dot(const scalarField& v1, const scalarField& v2)
{
    scalar s = 0;
    forAll(i, v1.size()) s += v1[i] * v2[i];
    return s;
}

}  // namespace UNAP

#endif
