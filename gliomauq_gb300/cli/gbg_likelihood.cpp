// gbg_likelihood: the `likelihood` program on libgbglioma, with the
// reference's file contract (source/Likelihood/source/HGG_Likelihood.cpp):
//   reads   LikelihoodInput.txt  (PETsigma2, PETscale, T1uc, T2uc, slope)
//           HGG_data.dat, PET_data.dat, T1_data.dat, T2_data.dat (Matrix::D3D)
//           Sphere.dat           (Matrix::D2D, npoints x 3, when selective)
//   writes  Likelihood.txt       (-log L, "%Lf \n")
// Flags as the reference: -selectivePoints (default 1), -stepPet (3), -stepTi (2).
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "../../include/gbglioma.h"
#include "matrix_file.hpp"

using gbgcli::Args;
using gbgcli::Matrix;

int main(int argc, char **argv) {
    Args args{argc, argv};
    gbg_lik_params p;
    {
        std::ifstream in("LikelihoodInput.txt");
        if (!(in >> p.pet_sigma2 >> p.pet_scale >> p.t1_uc >> p.t2_uc >> p.slope)) {
            std::printf("Aborting: missing input file LikelihoodInput.txt \n");
            std::abort();  // the reference aborts here (HGG_Likelihood.cpp:24-28)
        }
    }
    p.selective = args.as_int("-selectivePoints", 1) != 0;
    p.step_pet = args.as_int("-stepPet", 3);
    p.step_ti = args.as_int("-stepTi", 2);
    Matrix model, pet, t1, t2, pts;
    try {
        model = gbgcli::read_matrix("HGG_data.dat", 3);
        pet = gbgcli::read_matrix("PET_data.dat", 3);
        t1 = gbgcli::read_matrix("T1_data.dat", 3);
        t2 = gbgcli::read_matrix("T2_data.dat", 3);
        if (p.selective) pts = gbgcli::read_matrix("Sphere.dat", 2);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "gbg_likelihood: %s\n", e.what());
        return 1;
    }
    const int n = model.nx;
    if (model.ny != n || model.nz != n || pet.nx != n || pet.ny != n || pet.nz != n || t1.nx != n ||
        t1.ny != n || t1.nz != n || t2.nx != n || t2.ny != n || t2.nz != n) {
        std::fprintf(stderr, "gbg_likelihood: fields must be cubic and of one size\n");
        return 1;
    }
    gbg_config cfg = {n, GBG_PREC_F64, 0, 0};
    gbg_handle *h = nullptr;
    gbg_lik_result r;
    if (gbg_create(&cfg, &h) != GBG_OK || gbg_set_phi(h, model.data.data()) != GBG_OK ||
        gbg_set_observations(h, pet.data.data(), t1.data.data(), t2.data.data(),
                             p.selective ? pts.data.data() : nullptr, p.selective ? pts.nx : 0,
                             &p) != GBG_OK ||
        gbg_loglik(h, &r) != GBG_OK) {
        std::fprintf(stderr, "gbg_likelihood: %s\n", gbg_last_error());
        if (h) gbg_destroy(h);
        return 4;
    }
    gbg_destroy(h);
    std::printf("L_Pet=%f, L_T1=%f, L_T2 = %f \n", r.l_pet, r.l_t1, r.l_t2);
    std::printf("LogLike = %f \n", r.total);
    FILE *f = std::fopen("Likelihood.txt", "w");
    if (f) {
        std::fprintf(f, "%Lf \n", -(long double)r.total);
        std::fclose(f);
    }
    return 0;
}
