// Test-oracle harness: the reference's own bracketed alpha solver on given
// node data.
//
// Compiled against the reference headers by oracle/build_ref.py
// (build_bisection), with the deck oracle/ref_deck.in for one lattice. It is
// test infrastructure only: it produces the golden vectors of
// tests/golden/bisection/ and is never linked into the product library.
//
// For each node it places the pulled populations f_q and the non-equilibrium
// parts f_neq_q where the reference's functor reads them (the previous halo
// array at hSD::getIndex(iP - c_q, q), the next array at hSD::getIndex(iP, q);
// EntropicStep.h:15-63, Collision.h:227-241 stores f_neq in `next`) and calls
//   Bisection_NewtonRaphsonSolver(functor, tolerance, iterationMax, alphaR,
//                                 1.0, alphaMax)        (EntropicStep.h:142-220)
// exactly as ForcedBNR_ELBM::solveAlpha does (Collision.h:883-909), with the
// tolerance and iteration cap given on the command line.
//
// Usage: run <input.bin> <output.bin> <tolerance> <iterationMax>
//   input : float64 n, then n records of f[Q], f_neq[Q], alphaMax, alphaGuess
//   output: n records of alpha, converged (1.0 / 0.0)
#include "ref_deck.in"

#include "Commons.h"
#include "MPIInitializer.h"
#include "FFTWInitializer.h"
#include "MathVector.h"
#include "Routine.h"

#include <cstdio>
#include <cstdlib>
#include <vector>

int main(int argc, char** argv) {
  using namespace lbm;
  if (argc != 5) {
    std::fprintf(stderr, "usage: %s input.bin output.bin tolerance iterationMax\n", argv[0]);
    return 2;
  }
  const double tolerance = std::atof(argv[3]);
  const int iterationMax = std::atoi(argv[4]);
  FILE* fin = std::fopen(argv[1], "rb");
  double nd = 0.0;
  if (!fin || std::fread(&nd, sizeof nd, 1, fin) != 1) {
    std::fprintf(stderr, "cannot read %s\n", argv[1]);
    return 3;
  }
  const long n = (long)nd;
  const int Q = L::dimQ;
  const size_t rec = 2 * (size_t)Q + 2;
  std::vector<double> in((size_t)n * rec);
  if (std::fread(in.data(), sizeof(double), in.size(), fin) != in.size()) {
    std::fprintf(stderr, "short input %s\n", argv[1]);
    return 3;
  }
  std::fclose(fin);

  std::vector<double> previous((size_t)hSD::volume() * Q, 0.0), next(previous.size(), 0.0);
  const Position iP = L::halo();  // interior node: iP - c_q stays inside the halo domain
  std::vector<double> out((size_t)n * 2);
  for (long i = 0; i < n; ++i) {
    const double* r = in.data() + (size_t)i * rec;
    for (int q = 0; q < Q; ++q) {
      previous[hSD::getIndex(iP - uiL::celerity()[q], q)] = r[q];
      next[hSD::getIndex(iP, q)] = r[Q + q];
    }
    const double alphaMax = r[2 * Q];
    double alphaR = r[2 * Q + 1];
    EntropicStepFunctor<double> functor(next.data(), previous.data(), iP);
    const bool converged = Bisection_NewtonRaphsonSolver(functor, tolerance, iterationMax, alphaR,
                                                         1.0, alphaMax);
    out[2 * i] = alphaR;
    out[2 * i + 1] = converged ? 1.0 : 0.0;
  }
  FILE* fout = std::fopen(argv[2], "wb");
  if (!fout || std::fwrite(out.data(), sizeof(double), out.size(), fout) != out.size()) {
    std::fprintf(stderr, "cannot write %s\n", argv[2]);
    return 4;
  }
  std::fclose(fout);
  return 0;
}
