/* UNAP::lduMatrix (src/matrix/lduMatrix/lduMatrix.hpp:17-349): LDU storage
 * on the host with the reference's constructors, accessors and setters.
 * The matrix is symmetric when lower and upper are one object.  A copy of
 * it lives on the GPU from its first numerical use: SpMV, the
 * preconditioners, smoothers and solvers all run there through the C ABI.
 * Any call that hands out a modifiable array (the accessors, the SET_*
 * calls) marks that copy stale: the next numerical call uploads the
 * coefficients again, or rebuilds the device structure when the addressing
 * may have changed.  Arrays adopted with reUse are not freed by the matrix
 * (the reference deletes them). */
#ifndef LDUMATRIX_HPP
#define LDUMATRIX_HPP

#include <vector>

#include "unapMatrix.hpp"

namespace UNAP
{

class lduMatrix : public matrix
{
private:
    label nCells_;
    labelField *lowerAddrPtr_, *upperAddrPtr_;
    scalarField *lowerPtr_, *diagPtr_, *upperPtr_;
    bool ownLowerAddr_, ownUpperAddr_, ownLower_, ownDiag_, ownUpper_;
    mutable interfaces* interfacesPtr_;
    mutable bool ownInterfaces_;
    mutable labelField* losortPtr_;
    mutable labelField* ownerStartPtr_;
    mutable labelField* losortStartPtr_;
    // device copy: 0 = not built; topology or values possibly changed
    mutable long int handle_;
    mutable bool topoStale_, valuesStale_, uploadedSymm_;

    void init_()
    {
        nCells_ = -1;
        lowerAddrPtr_ = upperAddrPtr_ = NULL;
        lowerPtr_ = diagPtr_ = upperPtr_ = NULL;
        ownLowerAddr_ = ownUpperAddr_ = ownLower_ = ownDiag_ = ownUpper_ = false;
        interfacesPtr_ = NULL;
        ownInterfaces_ = false;
        losortPtr_ = ownerStartPtr_ = losortStartPtr_ = NULL;
        handle_ = 0;
        topoStale_ = valuesStale_ = true;
        uploadedSymm_ = false;
    }

    template <class F>
    static void put_(F*& slot, bool& own, const F& src, bool reUse)
    {
        if (slot && own && slot != &src) delete slot;
        if (reUse) {
            slot = const_cast<F*>(&src);
            own = false;
        } else {
            slot = new F(src);
            own = true;
        }
    }

    void dropLower_()
    {
        if (lowerPtr_ && ownLower_ && lowerPtr_ != upperPtr_) delete lowerPtr_;
        lowerPtr_ = NULL;
        ownLower_ = false;
    }

    void setCoeffs_(const scalarField& diag, const scalarField& upper, const scalarField& lower,
                    bool reUse)
    {
        nCells_ = diag.size();
        put_(diagPtr_, ownDiag_, diag, reUse);
        dropLower_();
        put_(upperPtr_, ownUpper_, upper, reUse);
        if (&lower == &upper) {
            lowerPtr_ = upperPtr_;
            ownLower_ = false;
        } else {
            put_(lowerPtr_, ownLower_, lower, reUse);
        }
        valuesStale_ = true;
    }

    void setTopo_(const labelField& lowerAddr, const labelField& upperAddr, bool reUse)
    {
        put_(lowerAddrPtr_, ownLowerAddr_, lowerAddr, reUse);
        put_(upperAddrPtr_, ownUpperAddr_, upperAddr, reUse);
        clearAddressing_();
        topoStale_ = true;
    }

    void clearAddressing_() const
    {
        delete losortPtr_;
        delete ownerStartPtr_;
        delete losortStartPtr_;
        losortPtr_ = ownerStartPtr_ = losortStartPtr_ = NULL;
    }

    static std::vector<int> ints_(const labelField& v, const char* what)
    {
        std::vector<int> o((size_t)v.size());
        for (label i = 0; i < v.size(); ++i) o[(size_t)i] = detail::to_int(v[i], what);
        return o;
    }

public:
    lduMatrix() { init_(); }

    lduMatrix(const label& nCells, const labelField& lowerAddr, const labelField& upperAddr,
              const scalarField& lower, const scalarField& diag, const scalarField& upper)
    {
        init_();
        nCells_ = nCells;
        setTopo_(lowerAddr, upperAddr, false);
        setCoeffs_(diag, upper, lower, false);
        nCells_ = nCells;
    }

    lduMatrix(const label& nCells, const labelField& lowerAddr, const labelField& upperAddr,
              const scalarField& lower, const scalarField& diag, const scalarField& upper,
              const bool reUse)
    {
        init_();
        setTopo_(lowerAddr, upperAddr, reUse);
        setCoeffs_(diag, upper, lower, reUse);
        nCells_ = nCells;
    }

    /* topology only; coefficients follow with setMatrixCoeffients */
    lduMatrix(const label& nCells, const labelField& lowerAddr, const labelField& upperAddr)
    {
        init_();
        setTopo_(lowerAddr, upperAddr, false);
        nCells_ = nCells;
    }

    lduMatrix(const label& nCells, const labelField& lowerAddr, const labelField& upperAddr,
              const bool reUse)
    {
        init_();
        setTopo_(lowerAddr, upperAddr, reUse);
        nCells_ = nCells;
    }

    lduMatrix(const lduMatrix&) = delete;
    lduMatrix& operator=(const lduMatrix&) = delete;

    ~lduMatrix()
    {
        if (handle_) unap_cuda_matrix_destroy(handle_);
        dropLower_();
        if (ownUpper_) delete upperPtr_;
        if (ownDiag_) delete diagPtr_;
        if (ownLowerAddr_) delete lowerAddrPtr_;
        if (ownUpperAddr_) delete upperAddrPtr_;
        if (ownInterfaces_) delete interfacesPtr_;
        clearAddressing_();
    }

    // accessors hand out modifiable arrays: the device copy is refreshed
    // before the next numerical call
    virtual labelField& lowerAddr() const
    {
        topoStale_ = true;
        clearAddressing_();
        return *lowerAddrPtr_;
    }
    virtual labelField& upperAddr() const
    {
        topoStale_ = true;
        clearAddressing_();
        return *upperAddrPtr_;
    }
    virtual scalarField& lower() const
    {
        valuesStale_ = true;
        return *lowerPtr_;
    }
    virtual scalarField& diag() const
    {
        valuesStale_ = true;
        return *diagPtr_;
    }
    virtual scalarField& upper() const
    {
        valuesStale_ = true;
        return *upperPtr_;
    }
    scalarField& diag()
    {
        valuesStale_ = true;
        return *diagPtr_;
    }

    void SET_lowerAddr(labelField& v)
    {
        put_(lowerAddrPtr_, ownLowerAddr_, v, false);
        clearAddressing_();
        topoStale_ = true;
    }
    void SET_upperAddr(labelField& v)
    {
        put_(upperAddrPtr_, ownUpperAddr_, v, false);
        clearAddressing_();
        topoStale_ = true;
    }
    /* on a symmetric matrix this makes it asymmetric */
    void SET_lower(scalarField& v)
    {
        if (symm()) {
            lowerPtr_ = NULL;
            ownLower_ = false;
        }
        put_(lowerPtr_, ownLower_, v, false);
        valuesStale_ = true;
    }
    void SET_lower(label newSize)
    {
        if (symm()) {
            lowerPtr_ = NULL;
            ownLower_ = false;
        }
        dropLower_();
        lowerPtr_ = new scalarField(newSize);
        ownLower_ = true;
        valuesStale_ = true;
    }
    void SET_upper(scalarField& v)
    {
        const bool s = symm() && upperPtr_;
        put_(upperPtr_, ownUpper_, v, false);
        if (s) lowerPtr_ = upperPtr_;
        valuesStale_ = true;
    }
    void SET_upper(label newSize)
    {
        const bool s = symm() && upperPtr_;
        if (ownUpper_) delete upperPtr_;
        upperPtr_ = new scalarField(newSize);
        ownUpper_ = true;
        if (s) lowerPtr_ = upperPtr_;
        valuesStale_ = true;
    }
    void SET_diag(scalarField& v)
    {
        put_(diagPtr_, ownDiag_, v, false);
        valuesStale_ = true;
    }
    void SET_diag(label newSize)
    {
        if (ownDiag_) delete diagPtr_;
        diagPtr_ = new scalarField(newSize);
        ownDiag_ = true;
        valuesStale_ = true;
    }
    void freeLower()
    {
        if (!symm()) {
            dropLower_();
            lowerPtr_ = upperPtr_;
            valuesStale_ = true;
        }
    }
    void setSymm()
    {
        if (upperPtr_) {
            dropLower_();
            lowerPtr_ = upperPtr_;
        } else if (lowerPtr_) {
            upperPtr_ = lowerPtr_;
            ownUpper_ = ownLower_;
            ownLower_ = false;
        }
        valuesStale_ = true;
    }

    virtual bool symm() const { return lowerPtr_ == upperPtr_; }
    virtual label size() const { return nCells_; }
    virtual label nCells() const { return nCells_; }
    void size(label n) { nCells_ = n; }

    /* Apsi = A psi on the GPU (lduMatrixSpMV.cpp:16-98, same per-row order) */
    virtual void spMV(scalarField& Apsi, const scalarField& psi) const
    {
        if (Apsi.size() != nCells_ || psi.size() != nCells_) {
            COUT << "ERROR in lduMatrix::spMV: vector size differs from nCells" << ENDL;
            ERROR_EXIT;
        }
        detail::check(unap_cuda_spmv_host(deviceHandle(), psi.values(), Apsi.values()), "spMV");
    }

    /* faces ordered by neighbour, stable in face order
     * (lduMatrix::calcLosort, lduMatrix.cpp:310-367) */
    const labelField& losortAddr() const
    {
        if (!losortPtr_) {
            const labelField& u = *upperAddrPtr_;
            const label nf = u.size();
            labelField start(nCells_ + 1, 0);
            forAll(f, nf) start[u[f] + 1]++;
            forAll(c, nCells_) start[c + 1] += start[c];
            losortPtr_ = new labelField(nf);
            forAll(f, nf) (*losortPtr_)[start[u[f]]++] = f;
        }
        return *losortPtr_;
    }

    /* first face of every owner; owners past the last face start at nFaces
     * (lduMatrix::calcOwnerStart, lduMatrix.cpp:269-296) */
    const labelField& ownerStartAddr() const
    {
        if (!ownerStartPtr_) {
            const labelField& l = *lowerAddrPtr_;
            const label nf = l.size();
            ownerStartPtr_ = new labelField(nCells_ + 1, nf);
            labelField& s = *ownerStartPtr_;
            s[0] = 0;
            label next = 1;
            forAll(f, nf)
            {
                while (next <= l[f]) s[next++] = f;
            }
        }
        return *ownerStartPtr_;
    }

    /* start of every neighbour in losort order; cells past the largest
     * neighbour keep 0 and the last entry is nFaces
     * (lduMatrix::calcLosortStart, lduMatrix.cpp:381-414) */
    const labelField& losortStartAddr() const
    {
        if (!losortStartPtr_) {
            const labelField& u = *upperAddrPtr_;
            const labelField& lo = losortAddr();
            const label nf = u.size();
            losortStartPtr_ = new labelField(nCells_ + 1, 0);
            labelField& s = *losortStartPtr_;
            label next = 0, cur = 0;
            forAll(f, nf)
            {
                const label nb = u[lo[f]];
                if (nb > cur) {
                    while (next <= nb) s[next++] = f;
                    cur = nb;
                }
            }
            s[nCells_] = nf;
        }
        return *losortStartPtr_;
    }

    virtual interfaces& matrixInterfaces() const
    {
        if (!interfacesPtr_) {
            interfacesPtr_ = new interfaces;
            ownInterfaces_ = true;
        }
        return *interfacesPtr_;
    }
    virtual void matrixInterfaces(interfaces& a)
    {
        if (ownInterfaces_) delete interfacesPtr_;
        interfacesPtr_ = &a;
        ownInterfaces_ = false;
    }
    void matrixInterfaces(const label)
    {
        if (!interfacesPtr_) matrixInterfaces();
    }
    /* one system per GPU: processor interfaces are accepted and carry no
     * coupling (a run with neighbours is told so) */
    void createInterfacesTopology(const label nNeiProcs, const label*, const label*, const label*)
    {
        if (nNeiProcs > 0)
            std::cerr << "UNAP (GB300): processor interfaces ignored: one system per GPU"
                      << std::endl;
    }
    void fillInterfacesCofficients(const label*, const scalar*) {}
    virtual void initInterfaces(const scalarField&) const {}
    virtual void updateInterfaces(scalarField&) const {}

    void setMatrixCoeffients(const scalarField& diag, const scalarField& upper,
                             const scalarField& lower)
    {
        setCoeffs_(diag, upper, lower, false);
    }
    void setMatrixCoeffients(const scalarField& diag, const scalarField& upper,
                             const scalarField& lower, const bool reUse)
    {
        setCoeffs_(diag, upper, lower, reUse);
    }
    void setMatrixTopology(const labelField& upperAddr, const labelField& lowerAddr,
                           const bool reUse)
    {
        setTopo_(lowerAddr, upperAddr, reUse);
    }
    void setMatrixTopology(const labelField& upperAddr, const labelField& lowerAddr)
    {
        setTopo_(lowerAddr, upperAddr, false);
    }

    /* The matrix's handle in the C ABI (unap_cuda.h), built or refreshed from
     * the host arrays as needed.  No counterpart in the reference. */
    long int deviceHandle() const
    {
        if (!lowerAddrPtr_ || !upperAddrPtr_ || !diagPtr_ || !upperPtr_ || !lowerPtr_) {
            COUT << "ERROR in lduMatrix: addressing or coefficients were never set" << ENDL;
            ERROR_EXIT;
        }
        const int n = detail::to_int(nCells_, "nCells");
        const int nf = detail::to_int(upperPtr_->size(), "nFaces");
        // new addressing or a change of symmetry: a new device structure
        if (handle_ && (topoStale_ || uploadedSymm_ != symm())) {
            unap_cuda_matrix_destroy(handle_);
            handle_ = 0;
        }
        const double* lo = symm() ? NULL : lowerPtr_->values();
        if (!handle_) {
            std::vector<int> l = ints_(*lowerAddrPtr_, "lowerAddr"),
                             u = ints_(*upperAddrPtr_, "upperAddr");
            detail::check(unap_cuda_matrix_create(&handle_, n, nf, l.data(), u.data(), lo,
                                                  diagPtr_->values(), upperPtr_->values()),
                          "lduMatrix upload");
            uploadedSymm_ = symm();
        } else if (valuesStale_) {
            detail::check(unap_cuda_matrix_set_values(handle_, diagPtr_->values(),
                                                      upperPtr_->values(), lo),
                          "lduMatrix coefficient upload");
        }
        topoStale_ = valuesStale_ = false;
        return handle_;
    }
};

}  // namespace UNAP

#endif
