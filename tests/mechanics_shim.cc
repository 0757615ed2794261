// C entry point over include/prismspf/utilities/mechanics.h for the host test of the Voigt
// stress product (compiled with g++ by tests/test_mechanics_host.py).
#include <prismspf/utilities/mechanics.h>

extern "C" void ms_stress3(const double* C, const double* e, double* s) {
  dealii::Tensor<2, 6, double> c;
  dealii::Tensor<1, 6, double> ee, ss;
  for (int i = 0; i < 6; ++i) {
    ee[i] = e[i];
    for (int j = 0; j < 6; ++j) c[i][j] = C[6 * i + j];
  }
  prismspf::Mechanics::compute_stress<3, double, double>(c, ee, ss);
  for (int i = 0; i < 6; ++i) s[i] = ss[i];
}

extern "C" void ms_stress2(const double* C, const double* e, double* s) {
  dealii::Tensor<2, 3, double> c;
  dealii::Tensor<1, 3, double> ee, ss;
  for (int i = 0; i < 3; ++i) {
    ee[i] = e[i];
    for (int j = 0; j < 3; ++j) c[i][j] = C[3 * i + j];
  }
  prismspf::Mechanics::compute_stress<2, double, double>(c, ee, ss);
  for (int i = 0; i < 3; ++i) s[i] = ss[i];
}
