/* UNAP::matrix and its nested interfaces (src/matrix/unapMatrix.hpp:9-373):
 * solverPerformance, agglomeration, solver, preconditioner, smoother. */
#ifndef UNAPMATRIX_HPP
#define UNAPMATRIX_HPP

#include "PtrList.hpp"
#include "interfaces.hpp"
#include "unapVector.hpp"

namespace UNAP
{

class matrix
{
public:
    virtual ~matrix() {}

    /* Apsi = A psi */
    virtual void spMV(scalarField& Apsi, const scalarField& psi) const = 0;
    /* number of equations */
    virtual label size() const = 0;
    virtual scalarField& diag() const = 0;
    virtual bool symm() const = 0;
    virtual interfaces& matrixInterfaces() const = 0;
    virtual void initInterfaces(const scalarField& psi) const = 0;
    virtual void updateInterfaces(scalarField& Apsi) const = 0;

    /* Result of a solve (unapMatrix.hpp:43-174, unapMatrixTest.cpp:3-97) */
    class solverPerformance
    {
    private:
        scalar initialResidual_;
        scalar finalResidual_;
        scalar previousResidual_;
        label noIterations_;
        bool converged_;
        bool singular_;

    public:
        solverPerformance()
            : initialResidual_(0), finalResidual_(0), previousResidual_(0), noIterations_(0),
              converged_(false), singular_(false)
        {
        }

        solverPerformance(const scalar iRes, const scalar fRes, const label nIter,
                          const bool converged, const bool singular)
            : initialResidual_(iRes), finalResidual_(fRes), previousResidual_(iRes),
              noIterations_(nIter), converged_(converged), singular_(singular)
        {
        }

        scalar initialResidual() const { return initialResidual_; }
        scalar& initialResidual() { return initialResidual_; }
        scalar finalResidual() const { return finalResidual_; }
        scalar& finalResidual() { return finalResidual_; }
        scalar previousResidual() const { return previousResidual_; }
        scalar& previousResidual() { return previousResidual_; }
        label nIterations() const { return noIterations_; }
        label& nIterations() { return noIterations_; }
        bool converged() const { return converged_; }
        bool singular() const { return singular_; }

        /* converged when the final residual is below the tolerance, or
         * (with a relative tolerance above SMALL) at most that fraction of
         * the initial one, after at least minIter iterations */
        bool checkConvergence(const scalar tolerance, const scalar relTolerance, const label iter,
                              const label minIter)
        {
            converged_ = (finalResidual_ < tolerance ||
                          (relTolerance > SMALL && finalResidual_ <= relTolerance * initialResidual_)) &&
                         iter >= minIter;
            return converged_;
        }

        bool checkConvergence(const scalar tolerance, const label iter, const label minIter)
        {
            converged_ = finalResidual_ < tolerance && iter >= minIter;
            return converged_;
        }

        bool checkConvergence(const scalar tolerance, const scalar relTolerance)
        {
            converged_ = finalResidual_ < tolerance ||
                         (relTolerance > SMALL && finalResidual_ <= relTolerance * initialResidual_);
            return converged_;
        }

        bool checkSingularity(const scalar residual)
        {
            singular_ = !(residual > SMALL);
            return singular_;
        }
    };

    /* a hierarchy of coarse matrices (unapMatrix.hpp:177-241) */
    class agglomeration
    {
    public:
        agglomeration() {}
        virtual ~agglomeration() {}

        virtual label size() const = 0;
        virtual const matrix& coarseMatrixLevels(const label leveli) const = 0;
        virtual const labelField& restrictAddressing(const label leveli) const = 0;
        virtual const labelField& faceRestrictAddressing(const label leveli) const = 0;
        virtual void agglomerateMatrix(const label fineLevelIndex) = 0;
        virtual void agglomerate(const scalarField& weights) = 0;
        virtual void SET_nCellsInCoarsestLevel(const label i) = 0;
        virtual void SET_maxLevels(const label i) = 0;

        /* coarse[C] = sum of the fine values of the cells of C */
        template <typename T>
        void restrictField(Vector<T>& cf, const Vector<T>& ff, const label fineLevelIndex) const
        {
            const labelField& map = restrictAddressing(fineLevelIndex);
            cf.SET_zero();
            forAll(i, ff.size()) cf[map[i]] += ff[i];
        }

        /* fine[i] = coarse value of i's cell */
        template <typename T>
        void prolongField(Vector<T>& ff, const Vector<T>& cf, const label coarseLevelIndex) const
        {
            const labelField& map = restrictAddressing(coarseLevelIndex);
            forAll(i, ff.size()) ff[i] = cf[map[i]];
        }

        /* coarse face values: sums of the fine faces that map to a face */
        template <typename T>
        void restrictFaceField(Vector<T>& cf, const Vector<T>& ff, const label fineLevelIndex) const
        {
            const labelField& map = faceRestrictAddressing(fineLevelIndex);
            cf.SET_zero();
            forAll(i, ff.size())
            {
                if (map[i] >= 0) cf[map[i]] += ff[i];
            }
        }
    };

    /* solver settings (unapMatrixSolver.cpp:3-42): maxIter 1000, minIter 0,
     * relTol 1e-6, tolerance 0 */
    class solver
    {
    protected:
        label maxIter_;
        label minIter_;
        scalar relTol_;
        scalar tolerance_;
        bool ifPrint_;

    public:
        solver() : maxIter_(1000), minIter_(0), relTol_(1e-6), tolerance_(0.0), ifPrint_(false) {}
        virtual ~solver() {}

        virtual solverPerformance solve(scalarField& x, const matrix& A,
                                        const scalarField& b) const = 0;

        /* ||source||_2 + SMALL */
        scalar normFactor(const scalarField& source) const { return source.SumSqrt() + SMALL; }

        inline label maxIter() const { return maxIter_; }
        inline label minIter() const { return minIter_; }
        inline scalar relTol() const { return relTol_; }
        inline scalar tolerance() const { return tolerance_; }
        inline bool ifPrint() const { return ifPrint_; }

        void SET_maxIter(label maxIter) { maxIter_ = maxIter; }
        void SET_minIter(label minIter) { minIter_ = minIter; }
        void SET_relTol(scalar relTol) { relTol_ = relTol; }
        void SET_tolerance(scalar tolerance) { tolerance_ = tolerance; }
        void SET_ifPrint(bool ifPrint) { ifPrint_ = ifPrint; }
    };

    /* preconditioner base: the identity (unapMatrixPrecond.cpp:4-17) */
    class preconditioner
    {
    private:
        mutable scalarField rDTemp_;

    public:
        virtual ~preconditioner() {}

        virtual void precondition(scalarField& wA, const scalarField& rA) const
        {
            forAll(i, wA.size()) wA[i] = rA[i];
        }

        virtual const scalarField& rD() const { return rDTemp_; }
    };

    class smoother
    {
    public:
        smoother() {}
        virtual ~smoother() {}
        virtual void smooth(scalarField& x, const matrix& A, const scalarField& b,
                            const label nSweeps) const = 0;
        virtual void init() const = 0;
    };
};

}  // namespace UNAP

#endif
