// Test doubles with the public members of the reference's BVP, Frontera,
// Nudo and Interfaz (BVP/BVP.hpp:17-28, BVP/Frontera.hpp:15-38,
// Mesh/Nudo.hpp:33-55, Mesh/Interfaz.hpp:14-37) that FeynmanKacSolverGPU
// reads, so the drop-in can be exercised where the reference's headers and
// their Eigen dependency are absent.  Only member names and meanings follow
// the reference; nothing here computes anything.
#pragma once
#include <map>
#include <vector>

namespace ref_like {

struct Vector2d {
  double v[2] = {0.0, 0.0};
  double& operator[](int i) { return v[i]; }
  const double& operator[](int i) const { return v[i]; }
};
struct MatrixXd {  // column-major, like Eigen's default
  int n = 0;
  std::vector<double> a;
  int rows() const { return n; }
  const double* data() const { return a.data(); }
};

typedef double (*pfescalar)(Vector2d);
typedef Vector2d (*pfvectorial)(Vector2d);
typedef double (*pfdistancia)(std::vector<double>, Vector2d, Vector2d&, Vector2d&);
typedef bool (*pftipo)(Vector2d);

struct Coeficiente_Escalar { pfescalar funcion = nullptr; };
struct Coeficiente_Vectorial { pfvectorial funcion = nullptr; };
struct Frontera {
  pfdistancia Distancia = nullptr;
  pftipo Absorbente = nullptr, Neumann = nullptr;
  std::vector<double> parametros;
};
struct BVP {
  Coeficiente_Escalar u, g, c, f;
  Coeficiente_Vectorial b, gradiente_u, F, mu;
  Frontera frontera_dominio, frontera_subdominio;
};
struct Nudo {
  bool frontera = false;
  int indice_global = 0;
  Vector2d posicion_cartesiana;
  double posicion_angular = 0.0;
  double B = 0.0;
  std::map<int, double> G;
};
struct Interfaz {
  int interior = 0;
  Vector2d centro;
  double radio = 0.0, c2 = 0.0;
  MatrixXd iPsi;
  std::vector<Nudo> nudos_circunferencia;
};

}  // namespace ref_like
