/* UNAP::lduAgglomeration (src/matrix/lduMatrix/lduAgglomeration/
 * lduAgglomeration.hpp, lduAgglomerate.cpp:4-271,
 * lduAgglomerationAddressing.cpp:8-178, lduAgglomerateMatrix.cpp:3-131):
 * pairwise face agglomeration by the given weights, levels kept while they
 * have at least nCellsInCoarsestLevel cells (default 50), at most
 * maxLevels (default 50).  agglomerate() builds the hierarchy through the
 * C ABI (the same one MGSolver's device hierarchy uses) and keeps each
 * level's addressing and coarse matrix on the host. */
#ifndef LDUAGGLOMERATION_HPP
#define LDUAGGLOMERATION_HPP

#include <vector>

#include "lduMatrix.hpp"

namespace UNAP
{

class lduAgglomeration : public matrix::agglomeration
{
private:
    label maxLevels_;
    label nCellsInCoarsestLevel_;
    labelField nCells_;
    label nCreatedLevels_;
    const lduMatrix& finestMatrix_;
    std::vector<lduMatrix*> coarse_;
    std::vector<labelField*> restrict_, faceRestrict_;
    scalarField weights_;
    bool agglomerated_;

    void clear_()
    {
        for (size_t i = 0; i < coarse_.size(); ++i) {
            delete coarse_[i];
            delete restrict_[i];
            delete faceRestrict_[i];
        }
        coarse_.clear();
        restrict_.clear();
        faceRestrict_.clear();
        nCreatedLevels_ = 0;
    }

    void level_check_(const label i) const
    {
        if (i < 0 || i >= nCreatedLevels_) {
            std::cerr << "UNAP (GB300): no agglomeration level " << i << std::endl;
            ERROR_EXIT;
        }
    }

public:
    explicit lduAgglomeration(const lduMatrix& A)
        : maxLevels_(50), nCellsInCoarsestLevel_(50), nCreatedLevels_(0), finestMatrix_(A),
          agglomerated_(false)
    {
    }
    lduAgglomeration(const lduAgglomeration&) = delete;
    lduAgglomeration& operator=(const lduAgglomeration&) = delete;
    virtual ~lduAgglomeration() { clear_(); }

    virtual void agglomerate(const scalarField& weights)
    {
        clear_();
        weights_ = weights;
        long int h = 0;
        detail::check(unap_cuda_agglomeration_create(
                          &h, finestMatrix_.deviceHandle(), weights.values(),
                          detail::to_int(nCellsInCoarsestLevel_, "nCellsInCoarsestLevel"),
                          detail::to_int(maxLevels_, "maxLevels")),
                      "lduAgglomeration::agglomerate");
        int nl = 0;
        detail::check(unap_cuda_agglomeration_size(h, &nl), "lduAgglomeration::agglomerate");
        nCells_.SET_size(nl);
        label nFinePrev = finestMatrix_.size();
        label nFineFaces = weights.size();
        for (int k = 0; k < nl; ++k) {
            int n = 0, nf = 0, symm = 0;
            detail::check(unap_cuda_agglomeration_level(h, k, &n, &nf, &symm, NULL, NULL, NULL,
                                                        NULL, NULL, NULL, NULL),
                          "lduAgglomeration::agglomerate");
            std::vector<int> ra((size_t)nFinePrev), fr((size_t)nFineFaces), l((size_t)nf),
                u((size_t)nf);
            scalarField diag(n), upper(nf), lower(nf);
            detail::check(unap_cuda_agglomeration_level(h, k, NULL, NULL, NULL, ra.data(),
                                                        fr.data(), l.data(), u.data(),
                                                        diag.values(), upper.values(),
                                                        lower.values()),
                          "lduAgglomeration::agglomerate");
            labelField* rl = new labelField(nFinePrev);
            labelField* fl = new labelField(nFineFaces);
            labelField la(nf), ua(nf);
            forAll(i, nFinePrev)(*rl)[i] = ra[(size_t)i];
            forAll(i, nFineFaces)(*fl)[i] = fr[(size_t)i];
            forAll(i, nf)
            {
                la[i] = l[(size_t)i];
                ua[i] = u[(size_t)i];
            }
            lduMatrix* M = symm ? new lduMatrix(n, la, ua, upper, diag, upper)
                                : new lduMatrix(n, la, ua, lower, diag, upper);
            coarse_.push_back(M);
            restrict_.push_back(rl);
            faceRestrict_.push_back(fl);
            nCells_[k] = n;
            nFinePrev = n;
            nFineFaces = nf;
        }
        unap_cuda_agglomeration_destroy(h);
        nCreatedLevels_ = nl;
        agglomerated_ = true;
    }

    virtual label size() const { return nCreatedLevels_; }
    virtual const lduMatrix& coarseMatrixLevels(const label leveli) const
    {
        level_check_(leveli);
        return *coarse_[(size_t)leveli];
    }
    lduMatrix& coarseMatrix(const label leveli) const
    {
        level_check_(leveli);
        return *coarse_[(size_t)leveli];
    }
    virtual const labelField& restrictAddressing(const label leveli) const
    {
        level_check_(leveli);
        return *restrict_[(size_t)leveli];
    }
    virtual const labelField& faceRestrictAddressing(const label leveli) const
    {
        level_check_(leveli);
        return *faceRestrict_[(size_t)leveli];
    }

    /* coarse coefficients of level fineLevelIndex + 1 from the current
     * finer matrix: the hierarchy is rebuilt with the same weights (the
     * pairing depends on the weights only, so the addressing is the same) */
    virtual void agglomerateMatrix(const label)
    {
        if (agglomerated_) agglomerate(scalarField(weights_));
    }

    virtual void SET_nCellsInCoarsestLevel(const label i) { nCellsInCoarsestLevel_ = i; }
    virtual void SET_maxLevels(const label i) { maxLevels_ = i; }
    /* Sunway-only reorderings of the reference: nothing to do here */
    void agglomerationReorderTopo() {}
    void agglConstructRSSIterator() {}

    /* settings and weights of the last agglomerate() (MGSolver builds its
     * device hierarchy from them); no counterpart in the reference */
    label nCellsInCoarsestLevel() const { return nCellsInCoarsestLevel_; }
    label maxLevels() const { return maxLevels_; }
    bool agglomerated() const { return agglomerated_; }
    const scalarField& weights() const { return weights_; }
    const lduMatrix& finestMatrix() const { return finestMatrix_; }
};

}  // namespace UNAP

#endif
