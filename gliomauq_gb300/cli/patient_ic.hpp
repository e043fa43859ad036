// Glioma_HG_UQ::_ic_PatientCase (source/Glioma/Glioma_HG_UQ.cpp:67-225)
// restated in a chosen Real type: the patient anatomy mapped onto the
// (bpd*16)^3 grid, normalised tissue fractions, and the smoothed-sphere
// tumour around the centre read from HGG_TumorIC.bin.
#pragma once
#include <algorithm>
#include <cmath>
#include <vector>

#include "matrix_file.hpp"

namespace gbgcli {

template <typename Real>
void initial_state(int bpd, const gbgcli::Matrix &GM, const gbgcli::Matrix &WM, const gbgcli::Matrix &CSF, const gbgcli::Matrix &T1,
                   const gbgcli::Matrix &T2, const Real tumor_ic[3], std::vector<double> &pw,
                   std::vector<double> &pg, std::vector<double> &phi, double &L) {
    const int bsx = GM.nx, bsy = GM.ny, bsz = GM.nz;
    const int bmax = std::max(bsx, std::max(bsy, bsz));
    L = bmax * 0.1;
    const double brainH = 1.0 / ((double)(bmax));
    const Real tumorRadius = 0.005;
    const Real smooth_sup = 2.;
    const int n = bpd * 16;
    const Real h = 1. / 128;  // hard-coded in the reference (:130)
    const Real iw = 1. / (smooth_sup * h);
    pw.assign((size_t)n * n * n, 0.0);
    pg.assign(pw.size(), 0.0);
    phi.assign(pw.size(), 0.0);
    const Real hb = (Real)(1.0 / n);  // BlockInfo::h, a power of two
    for (int gz = 0; gz < n; gz++)
        for (int gy = 0; gy < n; gy++)
            for (int gx = 0; gx < n; gx++) {
                // info.pos(x, ix, iy, iz) = origin + h*i in Real (exact here)
                const int gi[3] = {gx, gy, gz};
                double x[3];
                for (int d = 0; d < 3; ++d) {
                    const int blk = gi[d] / 16, i = gi[d] % 16;
                    const Real origin = (Real)(blk * (16.0 / n));
                    x[d] = (Real)(origin + hb * (Real)i);
                }
                int mx = (int)std::floor(x[0] / brainH), my = (int)std::floor(x[1] / brainH),
                    mz = (int)std::floor(x[2] / brainH);
                mx -= (int)((bmax - bsx) * 0.5);
                my -= (int)((bmax - bsy) * 0.5);
                mz -= (int)((bmax - bsz) * 0.5);
                Real PGt, PWt, Pcsf, PT1, PT2;
                if ((mx < 0 || mx >= bsx) || (my < 0 || my >= bsy) || (mz < 0 || mz >= bsz)) {
                    PGt = 0.; PWt = 0.; Pcsf = 0.; PT1 = 0.; PT2 = 0.;
                } else {
                    PGt = GM(mx, my, mz);
                    PWt = WM(mx, my, mz);
                    Pcsf = CSF(mx, my, mz);
                    PT1 = T1(mx, my, mz);
                    PT2 = T2(mx, my, mz);
                }
                const Real MRIsignal = PT1 + PT2;
                Pcsf = (MRIsignal > 0.) ? 0. : Pcsf;
                const double all = PWt + PGt + Pcsf;
                Real cell_pw = 0, cell_pg = 0, cell_phi = 0;
                if (all > 0) {
                    PGt = PGt / all;
                    PWt = PWt / all;
                    Pcsf = Pcsf / all;
                    Pcsf = (Pcsf > 0.1) ? 1. : Pcsf;
                    if (Pcsf < 1.) {
                        cell_pw = PWt / (Pcsf + PWt + PGt);
                        cell_pg = PGt / (Pcsf + PWt + PGt);
                    }
                }
                const Real p[3] = {(Real)(x[0] - tumor_ic[0]), (Real)(x[1] - tumor_ic[1]),
                                   (Real)(x[2] - tumor_ic[2])};
                const Real dist = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
                const Real psi = (dist - tumorRadius) * iw;
                if ((psi < -1) && ((PGt > 0.001) || (PWt > 0.001)))
                    cell_phi = 1.0;
                else if (((-1 <= psi) && (psi <= 1)) && ((PGt > 0) || (PWt > 0)))
                    cell_phi = 1.0 * 0.5 * (1 - psi - std::sin(M_PI * psi) / (M_PI));
                else
                    cell_phi = 0.0;
                const size_t g = (size_t)gx + (size_t)n * ((size_t)gy + (size_t)n * gz);
                pw[g] = cell_pw;
                pg[g] = cell_pg;
                phi[g] = cell_phi;
            }
}

}  // namespace gbgcli
