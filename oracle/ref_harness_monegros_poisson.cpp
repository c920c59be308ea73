// Test-only: fills a reference BVP with the Monegros problem with c = 0
// (BVPs/Monegros_Poisson.hpp, the problem of main_test_mpi.cpp).  That header
// defines the same inline names as BVPs/Monegros_Revamped.hpp with other
// bodies (Monegros_c, Monegros_f), so it is included inside a namespace of
// its own; the headers it includes itself are included first, at global
// scope, so that their include guards keep them out of the namespace.
#include <eigen3/Eigen/Core>
#include <math.h>
#include <iostream>
#include "BVP/BVP.hpp"

namespace monegros_poisson {
#include "BVPs/Monegros_Poisson.hpp"
}

void ref_fill_monegros_poisson(BVP& bvp) {
  using namespace monegros_poisson;
  bvp.u.Inicializa(Monegros_u);
  bvp.g.Inicializa(Monegros_g);
  bvp.c.Inicializa(Monegros_c);
  bvp.f.Inicializa(Monegros_f);
  bvp.sigma.Inicializa(Monegros_sigma);
  bvp.b.Inicializa(Monegros_b);
  bvp.F.Inicializa(Monegros_F);
}
