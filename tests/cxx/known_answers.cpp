// Known answers of the reference's own examples, through the UNAP C++ API
// (include/unap/) on the GPU: the 2x2 system of test/ex3.cpp (x = (2, -2)
// after one PCG iteration, with each LDU preconditioner) and the COO -> LDU
// arrays of test/ex8.cpp:31-37.  Prints one line per check; exits 1 on the
// first failure.
#include <cmath>
#include <cstdio>

#include "PBiCGStab.hpp"
#include "PCG.hpp"
#include "lduDICPrecond.hpp"
#include "lduDILUPrecond.hpp"
#include "lduDiagPrecond.hpp"
#include "lduMatrix.hpp"
#include "matrixConversion.hpp"

using namespace UNAP;

static int fail(const char* what)
{
    std::printf("FAIL %s\n", what);
    return 1;
}

static bool near(double a, double b) { return std::fabs(a - b) <= 1e-12 * (1.0 + std::fabs(b)); }

int main()
{
    // A = [3 2; 2 6], b = (2, -8): x = (2, -2)
    const label n = 2;
    scalarField b(n);
    b[0] = 2.0;
    b[1] = -8.0;
    labelField lowerAddr(1, 0), upperAddr(1, 1);
    scalarField lower(1, 2.0), upper(1, 2.0), diag(n);
    diag[0] = 3.0;
    diag[1] = 6.0;
    const lduMatrix A(n, lowerAddr, upperAddr, lower, diag, upper);
    const matrix* Am = &A;
    {
        lduDICPrecond P(A);
        PCG solver(P);
        scalarField x(n);
        matrix::solverPerformance perf = solver.solve(x, *Am, b);
        std::printf("pcg_dic iterations %d x0 %.17g x1 %.17g\n", (int)perf.nIterations(), x[0],
                    x[1]);
        if (perf.nIterations() != 1 || !near(x[0], 2.0) || !near(x[1], -2.0)) return fail("ex3 DIC");
    }
    {
        lduDiagPrecond P(A);
        PCG solver(P);
        scalarField x(n);
        solver.SET_relTol(1e-12);
        matrix::solverPerformance perf = solver.solve(x, A, b);
        std::printf("pcg_diag iterations %d converged %d\n", (int)perf.nIterations(),
                    (int)perf.converged());
        if (!perf.converged() || !near(x[0], 2.0) || !near(x[1], -2.0)) return fail("ex3 Diag");
    }
    {
        lduDILUPrecond P(A);
        PBiCGStab solver(P);
        scalarField x(n);
        matrix::solverPerformance perf = solver.solve(x, A, b);
        std::printf("bicgstab_dilu iterations %d\n", (int)perf.nIterations());
        if (!perf.converged() || !near(x[0], 2.0) || !near(x[1], -2.0)) return fail("ex3 DILU");
    }
    {
        // SpMV of the same matrix: A (1, 1) = (5, 8)
        scalarField x(n, 1.0), y(n);
        A.spMV(y, x);
        if (y[0] != 5.0 || y[1] != 8.0) return fail("spMV");
        std::printf("spmv ok\n");
    }
    {
        // test/ex8.cpp: 5x5 COO (0-based, row-major) to LDU
        int row[17] = {0, 0, 0, 0, 1, 1, 1, 2, 2, 2, 3, 3, 3, 4, 4, 4, 4};
        int col[17] = {0, 1, 3, 4, 0, 1, 2, 1, 2, 4, 0, 3, 4, 0, 2, 3, 4};
        double data[17] = {1.1, 1.2, 1.4, 1.5, 2.1, 2.2, 2.3, 3.2, 3.3,
                           3.5, 4.1, 4.4, 4.5, 5.1, 5.3, 5.4, 5.5};
        lduMatrix& L = coo2ldu(data, row, col, 5, 17, false);
        const int ua[6] = {1, 3, 4, 2, 4, 4}, la[6] = {0, 0, 0, 1, 2, 3};
        const double dg[5] = {1.1, 2.2, 3.3, 4.4, 5.5};
        const double up[6] = {1.2, 1.4, 1.5, 2.3, 3.5, 4.5}, lo[6] = {2.1, 4.1, 5.1, 3.2, 5.3, 5.4};
        for (int i = 0; i < 6; ++i)
            if (L.upperAddr()[i] != ua[i] || L.lowerAddr()[i] != la[i] || L.upper()[i] != up[i] ||
                L.lower()[i] != lo[i])
                return fail("ex8 faces");
        for (int i = 0; i < 5; ++i)
            if (L.diag()[i] != dg[i]) return fail("ex8 diag");
        std::printf("coo2ldu ok symm %d\n", (int)L.symm());
        delete &L;
    }
    {
        // reorderCOO of the same entries given row by row in reverse column
        // order gives the row-major, column-sorted order back
        int row[7] = {0, 0, 0, 1, 1, 2, 2};
        int col[7] = {2, 1, 0, 1, 0, 2, 1};
        double val[7] = {0.2, 0.1, 0.0, 1.1, 1.0, 2.2, 2.1};
        reorderCOO(val, row, col, 3, 7);
        const int ec[7] = {0, 1, 2, 0, 1, 1, 2};
        const double ev[7] = {0.0, 0.1, 0.2, 1.0, 1.1, 2.1, 2.2};
        for (int i = 0; i < 7; ++i)
            if (col[i] != ec[i] || val[i] != ev[i]) return fail("reorderCOO");
        std::printf("reorder ok\n");
    }
    std::printf("ALL OK\n");
    return 0;
}
