/* UNAP matrix conversion (src/tools/matrixConversion/matrixConversion.hpp,
 * matrixConversion.cpp:4-222, coo2ldu.cpp:3-148): COO and CSR input to an
 * lduMatrix, and the reorderings behind them, through the C ABI.  Indices
 * are 0-based. */
#ifndef MATRIXCONVERSION_HPP
#define MATRIXCONVERSION_HPP

#include <vector>

#include "lduMatrix.hpp"

namespace UNAP
{
namespace detail
{
inline std::vector<int> ints(const label* p, label n, const char* what)
{
    std::vector<int> o((size_t)n);
    for (label i = 0; i < n; ++i) o[(size_t)i] = to_int(p[i], what);
    return o;
}

/* the lduMatrix of a C ABI matrix handle (the handle is destroyed) */
inline lduMatrix& ldu_from_handle(long int h, const char* who)
{
    int n = 0, nf = 0, symm = 0;
    check(unap_cuda_matrix_size(h, &n, &nf, &symm), who);
    std::vector<int> l((size_t)nf), u((size_t)nf);
    scalarField lower(nf), diag(n), upper(nf);
    check(unap_cuda_matrix_get_ldu(h, l.data(), u.data(), lower.values(), diag.values(),
                                   upper.values()),
          who);
    unap_cuda_matrix_destroy(h);
    labelField la(nf), ua(nf);
    forAll(i, nf)
    {
        la[i] = l[(size_t)i];
        ua[i] = u[(size_t)i];
    }
    return symm ? *new lduMatrix(n, la, ua, upper, diag, upper)
                : *new lduMatrix(n, la, ua, lower, diag, upper);
}
}  // namespace detail

/* data[...] regrouped cell by cell: face i goes to its cell order[i]'s
 * block (cellFaces[c] faces per cell), in input order within a block
 * (matrixConversion.cpp:4-35) */
inline void sortData(scalarField& data, const labelField& order, const labelField& cellFaces)
{
    const label nCells = cellFaces.size();
    labelField next(nCells + 1, 0);
    forAll(c, nCells) next[c + 1] = next[c] + cellFaces[c];
    scalarField old(data);
    forAll(i, data.size()) data[next[order[i]]++] = old[i];
}

/* entries grouped by row, each row ordered by column; values move along */
inline void reorderCOO(scalar* dataPtr, label* rowsPtr, label* columnPtr, const label nCells,
                       const label size)
{
    std::vector<int> r = detail::ints(rowsPtr, size, "row"), c = detail::ints(columnPtr, size, "column");
    detail::check(unap_cuda_reorder_coo(dataPtr, r.data(), c.data(),
                                        detail::to_int(nCells, "nCells"),
                                        detail::to_int(size, "size")),
                  "reorderCOO");
    forAll(i, size)
    {
        rowsPtr[i] = r[(size_t)i];
        columnPtr[i] = c[(size_t)i];
    }
}

/* val[newOrder[i]] = old val[i] */
inline void reorderValue(scalar* val, const label* newOrder, const label size)
{
    std::vector<int> o = detail::ints(newOrder, size, "newOrder");
    detail::check(unap_cuda_reorder_value(val, o.data(), detail::to_int(size, "size")),
                  "reorderValue");
}

inline void reorder_faces_(bool byColumn, label* rowsPtr, label* columnPtr, const label nCells,
                           const label size, label* newOrder)
{
    std::vector<int> r = detail::ints(rowsPtr, size, "row"), c = detail::ints(columnPtr, size, "column"),
                     o((size_t)size);
    const int n = detail::to_int(nCells, "nCells"), s = detail::to_int(size, "size");
    detail::check(byColumn ? unap_cuda_reorder_lface(r.data(), c.data(), n, s, o.data())
                           : unap_cuda_reorder_uface(r.data(), c.data(), n, s, o.data()),
                  byColumn ? "reorderLFace" : "reorderUFace");
    forAll(i, size)
    {
        rowsPtr[i] = r[(size_t)i];
        columnPtr[i] = c[(size_t)i];
        newOrder[i] = o[(size_t)i];
    }
}

/* upper-side entries grouped by row and ordered by column; newOrder[i] is
 * entry i's new position */
inline void reorderUFace(label* rowsPtr, label* columnPtr, const label nCells, const label size,
                         label* newOrder)
{
    reorder_faces_(false, rowsPtr, columnPtr, nCells, size, newOrder);
}

/* lower-side entries grouped by column, stable in input order */
inline void reorderLFace(label* rowsPtr, label* columnPtr, const label nCells, const label size,
                         label* newOrder)
{
    reorder_faces_(true, rowsPtr, columnPtr, nCells, size, newOrder);
}

/* COO (0-based, grouped by row) of a structurally symmetric matrix to LDU;
 * symm says the values are symmetric.  The caller owns the new matrix. */
inline lduMatrix& coo2ldu(const scalar* dataPtr, const label* rowsPtr, const label* columnPtr,
                          const label nCells, const label size, const bool symm)
{
    std::vector<int> r((size_t)size), c((size_t)size);
    for (label i = 0; i < size; ++i) {
        r[(size_t)i] = detail::to_int(rowsPtr[i], "row") + 1;
        c[(size_t)i] = detail::to_int(columnPtr[i], "column") + 1;
    }
    const int n = detail::to_int(nCells, "nCells"), s = detail::to_int(size, "size"),
              sy = symm ? 1 : 0;
    long int h = 0;
    coo2ldumatrixcreat_(&h, dataPtr, r.data(), c.data(), &n, &s, &sy);
    if (!h) {
        std::cerr << "UNAP (GB300): coo2ldu failed: " << unap_cuda_last_error() << std::endl;
        ERROR_EXIT;
    }
    return detail::ldu_from_handle(h, "coo2ldu");
}

/* CSR (0-based row pointer of nCells + 1 entries, columns sorted per row) */
inline lduMatrix& csr2ldu(const scalar* dataPtr, const label* compRowsPtr, const label* columnPtr,
                          const label nCells, const label size, const bool symm)
{
    std::vector<int> r = detail::ints(compRowsPtr, nCells + 1, "row pointer"),
                     c = detail::ints(columnPtr, size, "column");
    const int n = detail::to_int(nCells, "nCells"), s = detail::to_int(size, "size"),
              sy = symm ? 1 : 0;
    long int h = 0;
    csr2ldumatrixcreat_(&h, dataPtr, r.data(), c.data(), &n, &s, &sy);
    if (!h) {
        std::cerr << "UNAP (GB300): csr2ldu failed: " << unap_cuda_last_error() << std::endl;
        ERROR_EXIT;
    }
    return detail::ldu_from_handle(h, "csr2ldu");
}

}  // namespace UNAP

#endif
