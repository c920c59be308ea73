// Test-only: fills a reference BVP with the Monegros problem with c = -1
// (BVPs/Monegros_Revamped.hpp).  Separate translation unit because the
// Monegros and Franke headers define inline functions with the same names.
#include "BVPs/Monegros_Revamped.hpp"
#include "BVP/BVP.hpp"

void ref_fill_monegros(BVP& bvp) {
  bvp.u.Inicializa(Monegros_u);
  bvp.g.Inicializa(Monegros_g);
  bvp.c.Inicializa(Monegros_c);
  bvp.f.Inicializa(Monegros_f);
  bvp.sigma.Inicializa(Monegros_sigma);
  bvp.b.Inicializa(Monegros_b);
  bvp.F.Inicializa(Monegros_F);
}
