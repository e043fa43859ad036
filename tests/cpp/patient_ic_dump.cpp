// Writes the restated initial density of a patient (gliomauq_gb300/cli/patient_ic.hpp)
// for 4^3 blocks to a Matrix::D3D file: argv = <anatomy base> <HGG_TumorIC.bin> <out>.
#include "patient_ic.hpp"
#include <cstdio>
int main(int argc, char** argv) {
  using namespace gbgcli;
  std::string base = argv[1];
  Matrix GM = read_matrix(base + "_GM.dat", 3), WM = read_matrix(base + "_WM.dat", 3), CSF = read_matrix(base + "_CSF.dat", 3), T1 = read_matrix(base + "_T1.dat", 3), T2 = read_matrix(base + "_T2.dat", 3);
  float ic[3]; FILE* f = fopen(argv[2], "rb"); if (fread(ic, 4, 3, f) != 3) return 3; fclose(f);
  std::vector<double> pw, pg, phi; double L;
  const float t[3] = {ic[0], ic[1], ic[2]};
  initial_state<float>(4, GM, WM, CSF, T1, T2, t, pw, pg, phi, L);
  write_d3d(argv[3], 64, 64, 64, phi);
}
