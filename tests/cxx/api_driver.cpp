// Drives every numerical call of the UNAP C++ API (include/unap/) on one
// system so a test can compare the results with the oracle: the natural-
// order 7-point Laplacian of an nx x ny x nz grid (faces sorted by owner,
// upper = lower = -1, diag = row sum of |offdiag| + shift), with b and x0
// read from a file of 2 n doubles.  Writes, as raw doubles: A x0; DIC w and
// rD for r = b; 2 Gauss-Seidel sweeps from x0; the Chebyshev estimate and
// one 3-sweep smooth after it from x0; PCG+DIC and PBiCGStab+DILU solves to
// relTol 1e-10 from 0 (iterations, then x); the agglomeration's level sizes;
// MGSolver with Gauss-Seidel and with Chebyshev smoothers to relTol 1e-8
// from 0 (iterations, then x).
//
//   api_driver nx ny nz shift in.bin out.bin
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "MG.hpp"
#include "PBiCGStab.hpp"
#include "PCG.hpp"
#include "lduDICPrecond.hpp"
#include "lduDILUPrecond.hpp"

using namespace UNAP;

static std::vector<double> out;

static void put(const scalarField& v)
{
    for (label i = 0; i < v.size(); ++i) out.push_back(v[i]);
}

int main(int argc, char** argv)
{
    if (argc != 7) {
        std::fprintf(stderr, "usage: api_driver nx ny nz shift in.bin out.bin\n");
        return 2;
    }
    const label nx = atoi(argv[1]), ny = atoi(argv[2]), nz = atoi(argv[3]);
    const double shift = atof(argv[4]);
    const label n = nx * ny * nz;
    std::vector<label> lv, uv;
    for (label c = 0; c < n; ++c) {
        const label i = c % nx, j = (c / nx) % ny, k = c / (nx * ny);
        if (i < nx - 1) lv.push_back(c), uv.push_back(c + 1);
        if (j < ny - 1) lv.push_back(c), uv.push_back(c + nx);
        if (k < nz - 1) lv.push_back(c), uv.push_back(c + nx * ny);
    }
    const label nf = (label)lv.size();
    labelField lowerAddr(lv.data(), nf), upperAddr(uv.data(), nf);
    scalarField upper(nf, -1.0), diag(n, 0.0);
    for (label f = 0; f < nf; ++f) {
        diag[lv[f]] += 1.0;
        diag[uv[f]] += 1.0;
    }
    for (label c = 0; c < n; ++c) diag[c] += shift;
    lduMatrix A(n, lowerAddr, upperAddr, upper, diag, upper);

    std::vector<double> in(2 * n);
    FILE* f = std::fopen(argv[5], "rb");
    if (!f || std::fread(in.data(), sizeof(double), in.size(), f) != in.size()) return 2;
    std::fclose(f);
    const scalarField b(in.data(), n), x0(in.data() + n, n);

    scalarField y(n);
    A.spMV(y, x0);
    put(y);

    lduDICPrecond dic(A);
    scalarField w(n);
    dic.precondition(w, b);
    put(w);
    put(dic.rD());

    lduGaussSeidelSmoother gs;
    scalarField x(x0);
    gs.smooth(x, A, b, 2);
    put(x);

    chebySmoother cs;
    x = x0;
    cs.smooth(x, A, b, 3);  // first call: the estimate only
    out.push_back(cs.maxEigenValue());
    put(x);
    cs.smooth(x, A, b, 3);
    put(x);

    {
        PCG solver(dic);
        solver.SET_relTol(1e-10);
        scalarField xs(n);
        matrix::solverPerformance p = solver.solve(xs, A, b);
        out.push_back(p.nIterations());
        put(xs);
    }
    {
        lduDILUPrecond dilu(A);
        PBiCGStab solver(dilu);
        solver.SET_relTol(1e-10);
        scalarField xs(n);
        matrix::solverPerformance p = solver.solve(xs, A, b);
        out.push_back(p.nIterations());
        put(xs);
    }

    // MGSolver on |upper| / ||upper|| weights, as the reference's MG entry
    // point normalizes them
    scalarField weights(nf);
    double nrm = 0;
    for (label i = 0; i < nf; ++i) nrm += upper[i] * upper[i];
    nrm = std::sqrt(nrm);
    for (label i = 0; i < nf; ++i) weights[i] = std::fabs(upper[i]) / nrm;
    lduAgglomeration aggl(A);
    aggl.agglomerate(weights);
    out.push_back(aggl.size());
    for (label k = 0; k < aggl.size(); ++k) out.push_back(aggl.coarseMatrixLevels(k).size());
    for (int kind = 1; kind <= 2; ++kind) {
        PtrList<matrix::smoother> sm(aggl.size() + 1);
        for (label k = 0; k <= aggl.size(); ++k) {
            if (kind == 1)
                sm.setLevel(k, *new lduGaussSeidelSmoother);
            else
                sm.setLevel(k, *new chebySmoother);
        }
        MGSolver mg(A, aggl, sm);
        mg.SET_relTol(1e-8);
        scalarField xs(n);
        matrix::solverPerformance p = mg.solve(xs, A, b);
        out.push_back(p.nIterations());
        put(xs);
    }

    f = std::fopen(argv[6], "wb");
    if (!f) return 2;
    std::fwrite(out.data(), sizeof(double), out.size(), f);
    std::fclose(f);
    std::printf("ok %zu doubles\n", out.size());
    return 0;
}
