// Accuracy of emcg::expTab (the Poisson residual's exp) against the host libm
// exp: prints the largest relative difference over a sweep of arguments and
// the results at the edges of the table-driven range.
#include <cmath>
#include <cstdio>
#include <random>

#include "emcg_exp.h"

int main() {
  double tab[emcg::kExpTab];
  for (int j = 0; j < emcg::kExpTab; j++)
    tab[j] = std::exp2(j / double(emcg::kExpTab));
  double worst = 0, worstX = 0;
  std::mt19937_64 g(7);
  std::uniform_real_distribution<double> u(-699.9, 699.9), s(-40.0, 40.0);
  for (int i = 0; i < 2000000; i++) {
    const double x = i & 1 ? u(g) : s(g);
    const double a = emcg::expTab(x, tab), b = std::exp(x);
    const double rel = std::fabs(a - b) / b;
    if (rel > worst) {
      worst = rel;
      worstX = x;
    }
  }
  for (double x : {0.0, -0.0, 1e-300, -1e-300, 0.5 * std::log(2.0) / emcg::kExpTab, 699.99, -699.99}) {
    const double rel = std::fabs(emcg::expTab(x, tab) - std::exp(x)) / std::exp(x);
    if (rel > worst) {
      worst = rel;
      worstX = x;
    }
  }
  const bool specials = std::isinf(emcg::expTab(800.0, tab)) && emcg::expTab(-800.0, tab) == 0.0 &&
                        std::isnan(emcg::expTab(NAN, tab)) && std::isinf(emcg::expTab(INFINITY, tab));
  std::printf("%.3e %.17g %d\n", worst, worstX, specials ? 1 : 0);
  return 0;
}
