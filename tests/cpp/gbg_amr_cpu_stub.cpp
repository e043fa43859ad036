// Test infrastructure only: a CPU stand-in for the gbg_amr_* entry points the
// drop-in back-end (include/gbglioma_blockprocessing.hpp) calls, so that its
// wiring can be driven on a machine without a GPU. It holds a uniform block
// grid (every block at one level, tiling the unit cube) and computes steps
// with the oracle's C restatement of the reference's RD step
// (oracle/gliomauq_oracle.c, orc_rd_step_f64 / orc_rd_step_f32ref). Grids with
// several levels are refused. Call counts are kept for the test.
#include <cstring>
#include <string>
#include <vector>

#include "gbglioma.h"
#include "gliomauq_oracle.h"

struct gbg_handle {
    int prec = 0, cap = 0, n = 0;
    std::vector<gbg_block> blocks;
    std::vector<double> pw, pg, phi;  // global x-fastest
};

namespace {
std::string g_err;
int g_calls[4];  // set_grid, build_ghosts, step, get_phi

size_t gidx(const gbg_block &b, int n, int c) {
    const int x = c % 16, y = (c / 16) % 16, z = c / 256;
    return (size_t)(b.ix * 16 + x) + (size_t)n * ((size_t)(b.iy * 16 + y) + (size_t)n * (b.iz * 16 + z));
}
}  // namespace

extern "C" {

int stub_calls(int i) { return g_calls[i]; }

const char *gbg_last_error(void) { return g_err.c_str(); }

int gbg_destroy(gbg_handle *h) {
    delete h;
    return GBG_OK;
}

int gbg_amr_create(const gbg_amr_config *cfg, gbg_handle **out) {
    if (!cfg || !out || cfg->max_blocks < 1) return GBG_ERR_ARG;
    gbg_handle *h = new gbg_handle;
    h->prec = cfg->precision;
    h->cap = cfg->max_blocks;
    *out = h;
    return GBG_OK;
}

int gbg_amr_set_grid(gbg_handle *h, int nb, const gbg_block *blocks, const double *pw, const double *pg,
                     const double *phi) {
    ++g_calls[0];
    if (nb < 1 || nb > h->cap) return GBG_ERR_ARG;
    const int level = blocks[0].level, side = 1 << level;
    if (nb != side * side * side) {
        g_err = "stub: uniform grids only";
        return GBG_ERR_UNSUPPORTED;
    }
    for (int b = 0; b < nb; ++b)
        if (blocks[b].level != level) {
            g_err = "stub: uniform grids only";
            return GBG_ERR_UNSUPPORTED;
        }
    h->n = 16 * side;
    const size_t N = (size_t)h->n * h->n * h->n;
    h->blocks.assign(blocks, blocks + nb);
    h->pw.assign(N, 0.0);
    h->pg.assign(N, 0.0);
    h->phi.assign(N, 0.0);
    for (int b = 0; b < nb; ++b)
        for (int c = 0; c < 4096; ++c) {
            const size_t g = gidx(blocks[b], h->n, c);
            h->pw[g] = pw[(size_t)b * 4096 + c];
            h->pg[g] = pg[(size_t)b * 4096 + c];
            h->phi[g] = phi[(size_t)b * 4096 + c];
        }
    return GBG_OK;
}

int gbg_amr_build_ghosts(gbg_handle *h) {
    ++g_calls[1];
    return h->n ? GBG_OK : GBG_ERR_STATE;
}

int gbg_amr_step(gbg_handle *h, double Dw, double Dg, double rho, double dt, long nsteps) {
    ++g_calls[2];
    const int n = h->n;
    const size_t N = (size_t)n * n * n;
    const double hh = 1.0 / n;
    for (long k = 0; k < nsteps; ++k) {
        if (h->prec == GBG_PREC_F64) {
            std::vector<double> out(N);
            orc_rd_step_f64(n, h->pw.data(), h->pg.data(), h->phi.data(), out.data(), Dw, Dg, rho, dt, hh, 1);
            h->phi.swap(out);
        } else {
            std::vector<float> pw(h->pw.begin(), h->pw.end()), pg(h->pg.begin(), h->pg.end()),
                phi(h->phi.begin(), h->phi.end()), out(N);
            orc_rd_step_f32ref(n, pw.data(), pg.data(), phi.data(), out.data(), (float)Dw, (float)Dg, (float)rho,
                               dt, hh, 1);
            h->phi.assign(out.begin(), out.end());
        }
    }
    return GBG_OK;
}

int gbg_amr_get_phi(gbg_handle *h, double *phi) {
    ++g_calls[3];
    for (size_t b = 0; b < h->blocks.size(); ++b)
        for (int c = 0; c < 4096; ++c) phi[b * 4096 + c] = h->phi[gidx(h->blocks[b], h->n, c)];
    return GBG_OK;
}

}  // extern "C"
