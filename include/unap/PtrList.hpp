/* UNAP::PtrList<T>: an owning list of pointers (src/base/PtrList/PtrList.hpp):
 * setLevel(i, obj) takes ownership of obj, the destructor deletes what the
 * list holds.  Not copyable (the elements may be abstract). */
#ifndef PTRLIST_HPP
#define PTRLIST_HPP

#include "unap.hpp"

namespace UNAP
{

template <typename T>
class PtrList
{
private:
    label size_;
    T** ptrs_;

    void clear()
    {
        if (!ptrs_) return;
        forAll(i, size_) delete ptrs_[i];
        delete[] ptrs_;
        ptrs_ = NULL;
    }

public:
    PtrList() : size_(50), ptrs_(new T*[50]()) {}
    explicit PtrList(const label size) : size_(size), ptrs_(new T*[size > 0 ? size : 1]()) {}
    PtrList(const PtrList<T>&) = delete;
    PtrList& operator=(const PtrList<T>&) = delete;
    ~PtrList() { clear(); }

    inline label size() const { return size_; }
    inline bool isEmpty() const { return size_ == 0; }

    /* resize; elements beyond the new size are deleted */
    void SET_size(const label newSize)
    {
        T** np = new T*[newSize > 0 ? newSize : 1]();
        forAll(i, size_)
        {
            if (i < newSize)
                np[i] = ptrs_[i];
            else
                delete ptrs_[i];
        }
        delete[] ptrs_;
        ptrs_ = np;
        size_ = newSize;
    }

    inline T& operator[](const label i) const { return *ptrs_[i]; }
    /* the element pointer (NULL where no element is set) */
    inline T* get(const label i) const { return (i >= 0 && i < size_) ? ptrs_[i] : NULL; }

    void setLevel(const label i, T& obj)
    {
        if (ptrs_[i] && ptrs_[i] != &obj) delete ptrs_[i];
        ptrs_[i] = &obj;
    }

    void removeLevel(const label i)
    {
        delete ptrs_[i];
        ptrs_[i] = NULL;
    }
};

}  // namespace UNAP

#endif
