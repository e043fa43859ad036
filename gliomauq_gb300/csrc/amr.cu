// Multiresolution block grid on the GPU: the RD step and the wavelet detail
// measure on MRAG's 16^3 blocks at mixed levels, with ghosts built from
// MRAG's ghost instruction tables.
//
// Layout in HBM: every field is block-major, 4096 cells per block, x fastest
// inside a block (the order of Block<...,16,16,16>::data). Ghost values of a
// block are stored in the order BlockLab::load visits them
// (source/MRAGcore/MRAGBlockLab.h:256-295): the 26 neighbour regions by code
// (x fastest, the centre skipped), each region z-y-x, for the stencil [-1, 2)
// per axis -- 1736 ghost cells per block.
//
// A ghost is sum_k value(src_k) * w_k in Real, starting from 0, terms in
// table order (BlockLab.h:286-291); w_k is the Real product of its three
// weights as BlockLab forms it (:289). The step is the Case2 operator and the
// Euler update of the uniform exact kernels, with the cell's face neighbours
// taken from the block or from its ghosts, h from the block's level, and the
// face diffusivities precomputed per cell and face from the same values
// (static between regrids). The FWT detail is BlockFWT::_fwt
// (source/MRAGcore/MRAGBlockFWT.h:219-298) with Interp2ndOrder filters on
// phi: for each of the 8^3 coarse points and each of the 7 detail subbands,
// the filter sum in the loop order of _filter, and the block's report is the
// largest magnitude (FWTReport::getOverAll_DetailMaxMag, :184-190).
//
// Compiled with -fmad=false: every operation rounds on its own.
#include <algorithm>
#include <utility>
#include <vector>

#include "gbg_internal.cuh"

namespace gbg {
namespace {

constexpr int BS = 16;
constexpr int BC = BS * BS * BS;  // cells per block
constexpr int NG = 1736;          // ghost cells per block, stencil [-1, 2)

// start of each of the 27 regions in the ghost list (region 13 is the block)
__host__ __device__ inline int region_start(int code) {
    int start = 0;
    for (int c = 0; c < code; ++c) {
        if (c == 13) continue;
        const int d0 = c % 3 - 1, d1 = (c / 3) % 3 - 1, d2 = (c / 9) % 3 - 1;
        const int n0 = d0 == 0 ? BS : 1, n1 = d1 == 0 ? BS : 1, n2 = d2 == 0 ? BS : 1;
        start += n0 * n1 * n2;
    }
    return start;
}

struct RegionTable {
    int start[27];
};

// ghost slot of lab coordinate (x, y, z), each in [-1, 16], not all inside
__device__ __forceinline__ int ghost_slot(const RegionTable &rt, int x, int y, int z) {
    const int d0 = x < 0 ? -1 : (x >= BS ? 1 : 0);
    const int d1 = y < 0 ? -1 : (y >= BS ? 1 : 0);
    const int d2 = z < 0 ? -1 : (z >= BS ? 1 : 0);
    const int code = (d0 + 1) + 3 * (d1 + 1) + 9 * (d2 + 1);
    const int n0 = d0 == 0 ? BS : 1, n1 = d1 == 0 ? BS : 1;
    const int lx = d0 == 0 ? x : 0, ly = d1 == 0 ? y : 0, lz = d2 == 0 ? z : 0;
    return rt.start[code] + lx + n0 * (ly + n1 * lz);
}

template <typename Real>
__global__ void k_ghost_eval(int nb, const long *__restrict__ start, const int *__restrict__ src_block,
                             const int *__restrict__ src_cell, const double *__restrict__ w,
                             const Real *__restrict__ field, Real *__restrict__ ghost) {
    const long total = (long)nb * NG;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        Real acc = (Real)0;
        for (long k = start[i]; k < start[i + 1]; ++k) {
            const Real v = field[(size_t)src_block[k] * BC + src_cell[k]];
            acc = acc + v * (Real)w[k];
        }
        ghost[i] = acc;
    }
}

// value of `field` at lab coordinate (x, y, z) of block b
template <typename Real>
__device__ __forceinline__ Real lab_at(const RegionTable &rt, const Real *field, const Real *ghost, int b,
                                       int x, int y, int z) {
    if (x >= 0 && x < BS && y >= 0 && y < BS && z >= 0 && z < BS)
        return field[(size_t)b * BC + x + BS * (y + BS * z)];
    return ghost[(size_t)b * NG + ghost_slot(rt, x, y, z)];
}

// per cell: brain sum b0 and the six face diffusivities df[0..5] (W E S N B F)
template <typename Real>
__global__ void k_amr_tables(int nb, RegionTable rt, const Real *__restrict__ pw, const Real *__restrict__ pg,
                             const Real *__restrict__ gpw, const Real *__restrict__ gpg, Real Dw, Real Dg,
                             Real *__restrict__ b0, double *__restrict__ df) {
    const long total = (long)nb * BC;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int b = (int)(i / BC), c = (int)(i % BC);
        const int x = c % BS, y = (c / BS) % BS, z = c / (BS * BS);
        const int nx[7] = {x, x - 1, x + 1, x, x, x, x};
        const int ny[7] = {y, y, y, y - 1, y + 1, y, y};
        const int nz[7] = {z, z, z, z, z, z - 1, z + 1};
        double inv[7];
        for (int k = 0; k < 7; ++k) {
            const Real a = lab_at(rt, pw, gpw, b, nx[k], ny[k], nz[k]);
            const Real g = lab_at(rt, pg, gpg, b, nx[k], ny[k], nz[k]);
            const Real brain = a + g;
            const Real kk = (a * Dw + g * Dg) / brain;
            inv[k] = 1.0 / (double)kk;
            if (k == 0) b0[i] = brain;
        }
        for (int f = 0; f < 6; ++f) df[(size_t)i * 6 + f] = 2.0 * (1.0 / (inv[0] + inv[f + 1]));
    }
}

__device__ __forceinline__ double reaction(double rho, double p) { return rho * p * (1. - p); }
__device__ __forceinline__ double reaction(float rho, float p) {
    const float rp = rho * p;
    return (double)rp * (1. - (double)p);
}

template <typename Real>
__global__ void k_amr_step(int nb, RegionTable rt, const int *__restrict__ level, const Real *__restrict__ phi,
                           const Real *__restrict__ gphi, const Real *__restrict__ b0,
                           const double *__restrict__ df, Real *__restrict__ out, Real rho, double dt) {
    const long total = (long)nb * BC;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int b = (int)(i / BC), c = (int)(i % BC);
        const int x = c % BS, y = (c / BS) % BS, z = c / (BS * BS);
        // h = info.h[0] is Real: 1 / (2^level * 16), a power of two
        const Real hR = (Real)1 / (Real)((1 << level[b]) * BS);
        const double h = (double)hR;
        const double ih2 = 1. / (h * h);
        const Real p0 = phi[i];
        const Real pW = lab_at(rt, phi, gphi, b, x - 1, y, z), pE = lab_at(rt, phi, gphi, b, x + 1, y, z);
        const Real pS = lab_at(rt, phi, gphi, b, x, y - 1, z), pN = lab_at(rt, phi, gphi, b, x, y + 1, z);
        const Real pB = lab_at(rt, phi, gphi, b, x, y, z - 1), pF = lab_at(rt, phi, gphi, b, x, y, z + 1);
        double d0 = 0.0, d1 = 0.0, d2 = 0.0, d3 = 0.0, d4 = 0.0, d5 = 0.0;
        const Real tissue = b0[i] + p0;
        if (tissue > 0.) {
            const double *t = df + (size_t)i * 6;
            d0 = t[0]; d1 = t[1]; d2 = t[2]; d3 = t[3]; d4 = t[4]; d5 = t[5];
        }
        if (d0 == 0 && pW > 0.) d1 *= 2.0;
        if (d1 == 0 && pE > 0.) d0 *= 2.0;
        if (d2 == 0 && pS > 0.) d3 *= 2.0;
        if (d3 == 0 && pN > 0.) d2 *= 2.0;
        if (d4 == 0 && pB > 0.) d5 *= 2.0;
        if (d5 == 0 && pF > 0.) d4 *= 2.0;
        const double fin = ih2 * (d0 * (double)pW + d1 * (double)pE + d2 * (double)pS + d3 * (double)pN +
                                  d4 * (double)pB + d5 * (double)pF);
        const double fout = -((d0 + d1 + d2 + d3 + d4 + d5) * (double)p0 * ih2);
        const double react = reaction(rho, p0);
        const Real dphidt = (Real)(fout + fin + react);
        Real v = (Real)((double)p0 + dt * (double)dphidt);
        v = ((Real)0 < v) ? v : (Real)0;
        v = (v < (Real)1) ? v : (Real)1;
        out[i] = v;
    }
}

// ---- fast FP32 mode (GBG_PREC_F32 handles) ------------------------------------
// The uniform fast path's arithmetic on the block grid: unit face
// coefficients c_f = 2 k_c k_n / (k_c + k_n), k = (p_w + r p_g) / (p_w + p_g)
// (double, rounded to float), a tissue mask (cell and its six lab
// neighbours have tissue), and per step
//   phi' = m * clamp(phi + a_l sum_f c_f (phi_f - phi) + b phi (1 - phi), 0, 1)
// in float, faces in the order W E S N B F, a_l = dt Dw / h_l^2 per block
// level. On a one-level grid this is the uniform fast path bit for bit.
// Table per cell: 7 floats (c_W, c_E, c_S, c_N, c_B, c_F, mask).
__global__ void k_amr_fast_tables(int nb, RegionTable rt, const float *__restrict__ pw, const float *__restrict__ pg,
                                  const float *__restrict__ gpw, const float *__restrict__ gpg, double ratio,
                                  float *__restrict__ tab) {
    const long total = (long)nb * BC;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int b = (int)(i / BC), c = (int)(i % BC);
        const int x = c % BS, y = (c / BS) % BS, z = c / (BS * BS);
        const int nx[7] = {x, x - 1, x + 1, x, x, x, x};
        const int ny[7] = {y, y, y, y - 1, y + 1, y, y};
        const int nz[7] = {z, z, z, z, z, z - 1, z + 1};
        double k[7];
        bool all = true;
        for (int q = 0; q < 7; ++q) {
            const double a = (double)lab_at(rt, pw, gpw, b, nx[q], ny[q], nz[q]);
            const double g = (double)lab_at(rt, pg, gpg, b, nx[q], ny[q], nz[q]);
            const double br = a + g;
            all = all && (br > 0.0);
            k[q] = br > 0.0 ? (a + ratio * g) / br : 0.0;
        }
        float *t = tab + (size_t)i * 7;
        for (int f = 0; f < 6; ++f) {
            // the face's two cells in the uniform tables' order: (cell, +neighbour)
            const bool minus = (f % 2) == 0;
            const double k0 = minus ? k[f + 1] : k[0], k1 = minus ? k[0] : k[f + 1];
            const double sum = k0 + k1;
            t[f] = (k0 > 0.0 && k1 > 0.0 && sum > 0.0) ? (float)(2.0 * k0 * k1 / sum) : 0.0f;
        }
        t[6] = all ? 1.0f : 0.0f;
    }
}

// One CTA per block: the block and its ghosts go to an 18^3 lab in shared
// memory, then 256 threads update 16 cells each.
__global__ void __launch_bounds__(256) k_amr_fast_step(int nb, RegionTable rt, const int *__restrict__ level,
                                                       const float *__restrict__ phi,
                                                       const float *__restrict__ gphi,
                                                       const float *__restrict__ tab, float *__restrict__ out,
                                                       double Dw, double rho, double dt) {
    constexpr int LS = BS + 2;
    __shared__ float lab[LS * LS * LS];
    for (int b = blockIdx.x; b < nb; b += gridDim.x) {
        __syncthreads();
        const float *pb = phi + (size_t)b * BC;
        const float *gb = gphi + (size_t)b * NG;
        for (int l = threadIdx.x; l < LS * LS * LS; l += blockDim.x) {
            const int x = l % LS - 1, y = (l / LS) % LS - 1, z = l / (LS * LS) - 1;
            const bool inside = x >= 0 && x < BS && y >= 0 && y < BS && z >= 0 && z < BS;
            lab[l] = inside ? pb[x + BS * (y + BS * z)] : gb[ghost_slot(rt, x, y, z)];
        }
        __syncthreads();
        const double h = 1.0 / (double)((1 << level[b]) * BS);
        const float a = (float)(dt * Dw * (1. / (h * h)));
        const float bb = (float)(dt * rho);
        for (int c = threadIdx.x; c < BC; c += blockDim.x) {
            const int x = c % BS, y = (c / BS) % BS, z = c / (BS * BS);
            const int l = (x + 1) + LS * ((y + 1) + LS * (z + 1));
            const float f0 = lab[l];
            const float *t = tab + ((size_t)b * BC + c) * 7;
            float lap = t[0] * (lab[l - 1] - f0);
            lap = fmaf(t[1], lab[l + 1] - f0, lap);
            lap = fmaf(t[2], lab[l - LS] - f0, lap);
            lap = fmaf(t[3], lab[l + LS] - f0, lap);
            lap = fmaf(t[4], lab[l - LS * LS] - f0, lap);
            lap = fmaf(t[5], lab[l + LS * LS] - f0, lap);
            float v = fmaf(a, lap, f0);
            v = fmaf(bb * f0, 1.0f - f0, v);
            v = fminf(fmaxf(v, 0.0f), 1.0f);
            out[(size_t)b * BC + c] = t[6] != 0.0f ? v : 0.0f;
        }
    }
}

// ---- fast FP32 mode, fused form (the default) -------------------------------
// The same arithmetic with less traffic per step: the ghosts are evaluated
// while the lab is filled (no ghost array written and read back), from the
// tables in 32-bit form, and the face coefficients are stored once per face
// (a cell's W face is its west neighbour's E face, formed from the same two
// cells in the same order) with a byte mask: 13,056 floats + 4096 bytes per
// block in place of 28,672 floats.
constexpr int NFX = (BS + 1) * BS * BS;  // faces per direction and block

__global__ void k_compact_tables(long ng, long ne, const long *__restrict__ start, const int *__restrict__ sb,
                                 const int *__restrict__ sc, const double *__restrict__ w, int *__restrict__ start32,
                                 int *__restrict__ src32, float *__restrict__ w32) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i <= ng || i < ne;
         i += (long)gridDim.x * blockDim.x) {
        if (i <= ng) start32[i] = (int)start[i];
        if (i < ne) {
            src32[i] = sb[i] * BC + sc[i];
            w32[i] = (float)w[i];  // the Real weight k_ghost_eval applies
        }
    }
}

// lab index (18^3, x fastest) of ghost slot g
__device__ __forceinline__ int ghost_lab(const RegionTable &rt, int g) {
    int code = 0;
    for (int c = 0; c < 27; ++c)
        if (c != 13 && rt.start[c] <= g) code = c;
    const int d0 = code % 3 - 1, d1 = (code / 3) % 3 - 1, d2 = code / 9 - 1;
    const int n0 = d0 == 0 ? BS : 1, n1 = d1 == 0 ? BS : 1;
    const int local = g - rt.start[code];
    const int lx = local % n0, ly = (local / n0) % n1, lz = local / (n0 * n1);
    const int x = d0 == 0 ? lx : (d0 < 0 ? -1 : BS), y = d1 == 0 ? ly : (d1 < 0 ? -1 : BS),
              z = d2 == 0 ? lz : (d2 < 0 ? -1 : BS);
    return (x + 1) + (BS + 2) * ((y + 1) + (BS + 2) * (z + 1));
}

__device__ __forceinline__ double fast_k(const RegionTable &rt, const float *pw, const float *gpw, const float *pg,
                                         const float *gpg, double ratio, int b, int x, int y, int z, bool &tissue) {
    const double a = (double)lab_at(rt, pw, gpw, b, x, y, z);
    const double g = (double)lab_at(rt, pg, gpg, b, x, y, z);
    const double br = a + g;
    tissue = br > 0.0;
    return tissue ? (a + ratio * g) / br : 0.0;
}

// per block: fx[x + 17 (y + 16 z)] (x in [0, 16], the face between x - 1 and
// x), fy[x + 16 (y + 17 z)], fz[x + 16 (y + 16 z)], z in [0, 16]; the mask
__global__ void k_amr_fast_faces(int nb, RegionTable rt, const float *__restrict__ pw, const float *__restrict__ pg,
                                 const float *__restrict__ gpw, const float *__restrict__ gpg, double ratio,
                                 float *__restrict__ fx, float *__restrict__ fy, float *__restrict__ fz,
                                 unsigned char *__restrict__ mask) {
    const long per = 3L * NFX + BC;
    const long total = (long)nb * per;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int b = (int)(i / per);
        const int r = (int)(i % per);
        bool t0, t1;
        if (r < 3 * NFX) {
            const int dir = r / NFX, f = r % NFX;
            int x, y, z, dx = 0, dy = 0, dz = 0;
            if (dir == 0) {
                x = f % (BS + 1), y = (f / (BS + 1)) % BS, z = f / ((BS + 1) * BS), dx = 1;
            } else if (dir == 1) {
                x = f % BS, y = (f / BS) % (BS + 1), z = f / (BS * (BS + 1)), dy = 1;
            } else {
                x = f % BS, y = (f / BS) % BS, z = f / (BS * BS), dz = 1;
            }
            // the face's two cells, minus side first (the tables' (cell, +neighbour) order)
            const double k0 = fast_k(rt, pw, gpw, pg, gpg, ratio, b, x - dx, y - dy, z - dz, t0);
            const double k1 = fast_k(rt, pw, gpw, pg, gpg, ratio, b, x, y, z, t1);
            const double sum = k0 + k1;
            const float c = (k0 > 0.0 && k1 > 0.0 && sum > 0.0) ? (float)(2.0 * k0 * k1 / sum) : 0.0f;
            float *dst = dir == 0 ? fx : (dir == 1 ? fy : fz);
            dst[(size_t)b * NFX + f] = c;
        } else {
            const int c = r - 3 * NFX;
            const int x = c % BS, y = (c / BS) % BS, z = c / (BS * BS);
            const int nx[7] = {x, x - 1, x + 1, x, x, x, x};
            const int ny[7] = {y, y, y, y - 1, y + 1, y, y};
            const int nz[7] = {z, z, z, z, z, z - 1, z + 1};
            bool all = true;
            for (int q = 0; q < 7; ++q) {
                fast_k(rt, pw, gpw, pg, gpg, ratio, b, nx[q], ny[q], nz[q], t0);
                all = all && t0;
            }
            mask[(size_t)b * BC + c] = all ? 1 : 0;
        }
    }
}

// One CTA per block: the block's cells and its ghosts (evaluated from the
// tables in slot order, as k_ghost_eval does) into an 18^3 lab, then 256
// threads update 16 cells each with the per-face coefficients. Launched with
// 256 threads (the loops' strides).
__global__ void __launch_bounds__(256) k_amr_fast_step_fused(int nb, RegionTable rt, const int *__restrict__ level,
                                                             const float *__restrict__ phi,
                                                             const int *__restrict__ gstart,
                                                             const int *__restrict__ gsrc,
                                                             const float *__restrict__ gw,
                                                             const float *__restrict__ fx,
                                                             const float *__restrict__ fy,
                                                             const float *__restrict__ fz,
                                                             const unsigned char *__restrict__ mask,
                                                             float *__restrict__ out, double Dw, double rho,
                                                             double dt) {
    constexpr int LS = BS + 2;
    __shared__ float lab[LS * LS * LS];
    for (int b = blockIdx.x; b < nb; b += gridDim.x) {
        __syncthreads();
        const float *pb = phi + (size_t)b * BC;
#pragma unroll 8
        for (int j = 0; j < BC / 256; ++j) {
            const int c = threadIdx.x + 256 * j;
            const int x = c % BS, y = (c / BS) % BS, z = c / (BS * BS);
            lab[(x + 1) + LS * ((y + 1) + LS * (z + 1))] = pb[c];
        }
        // the thread's ghosts (at most kGhostsPerThread) with their loads
        // batched: all offsets, then every first term's source and weight,
        // then those sources, then any further terms -- each ghost's sum
        // still starts from 0 and adds its terms in table order
        {
            constexpr int kG = (NG + 255) / 256;
            int st[kG], en[kG], s0[kG];
            float w0[kG], acc[kG];
#pragma unroll
            for (int j = 0; j < kG; ++j) {
                const int g = threadIdx.x + 256 * j;
                const long i = (long)b * NG + (g < NG ? g : 0);
                st[j] = g < NG ? gstart[i] : 0;
                en[j] = g < NG ? gstart[i + 1] : 0;
            }
#pragma unroll
            for (int j = 0; j < kG; ++j) {
                s0[j] = st[j] < en[j] ? gsrc[st[j]] : 0;
                w0[j] = st[j] < en[j] ? gw[st[j]] : 0.0f;
            }
#pragma unroll
            for (int j = 0; j < kG; ++j) acc[j] = st[j] < en[j] ? 0.0f + phi[s0[j]] * w0[j] : 0.0f;
#pragma unroll
            for (int j = 0; j < kG; ++j) {
                for (int k = st[j] + 1; k < en[j]; ++k) acc[j] = acc[j] + phi[gsrc[k]] * gw[k];
                const int g = threadIdx.x + 256 * j;
                if (g < NG) lab[ghost_lab(rt, g)] = acc[j];
            }
        }
        __syncthreads();
        const double h = 1.0 / (double)((1 << level[b]) * BS);
        const float a = (float)(dt * Dw * (1. / (h * h)));
        const float bb = (float)(dt * rho);
        const float *fxb = fx + (size_t)b * NFX, *fyb = fy + (size_t)b * NFX, *fzb = fz + (size_t)b * NFX;
        const unsigned char *mb = mask + (size_t)b * BC;
#pragma unroll 4
        for (int j = 0; j < BC / 256; ++j) {
            const int c = threadIdx.x + 256 * j;
            const int x = c % BS, y = (c / BS) % BS, z = c / (BS * BS);
            const int l = (x + 1) + LS * ((y + 1) + LS * (z + 1));
            const float f0 = lab[l];
            const int ix = x + (BS + 1) * (y + BS * z), iy = x + BS * (y + (BS + 1) * z), iz = c;
            float lap = fxb[ix] * (lab[l - 1] - f0);
            lap = fmaf(fxb[ix + 1], lab[l + 1] - f0, lap);
            lap = fmaf(fyb[iy], lab[l - LS] - f0, lap);
            lap = fmaf(fyb[iy + BS], lab[l + LS] - f0, lap);
            lap = fmaf(fzb[iz], lab[l - LS * LS] - f0, lap);
            lap = fmaf(fzb[iz + BS * BS], lab[l + LS * LS] - f0, lap);
            float v = fmaf(a, lap, f0);
            v = fmaf(bb * f0, 1.0f - f0, v);
            v = fminf(fmaxf(v, 0.0f), 1.0f);
            out[(size_t)b * BC + c] = mb[c] ? v : 0.0f;
        }
    }
}

// One CTA per block, one thread per coarse point (8^3 = 512): the seven
// detail subbands, then a max-reduction of their magnitudes.
template <typename Real>
__global__ void __launch_bounds__(512) k_amr_fwt(int nb, RegionTable rt, const Real *__restrict__ phi,
                                                 const Real *__restrict__ gphi, double *__restrict__ detail) {
    const int b = blockIdx.x;
    const int t = threadIdx.x;
    const int dx = t % 8, dy = (t / 8) % 8, dz = t / 64;
    // Interp2ndOrder: Ha = {1} on [0,1), Ga = {-0.5, 1, -0.5} on [-2,1)
    const Real ga[3] = {(Real)-0.5, (Real)1., (Real)-0.5};
    double mx = 0.0;
    for (int sb = 1; sb < 8; ++sb) {
        const int wx = sb & 1, wy = (sb >> 1) & 1, wz = (sb >> 2) & 1;
        const int s0 = wx ? -2 : 0, e0 = wx ? 1 : 1;
        const int s1 = wy ? -2 : 0, e1 = wy ? 1 : 1;
        const int s2 = wz ? -2 : 0, e2 = wz ? 1 : 1;
        Real result = 0;
        for (int iz = s2; iz < e2; iz++) {
            const Real wZ = wz ? ga[iz + 2] : (Real)1;
            for (int iy = s1; iy < e1; iy++) {
                const Real wY = wy ? ga[iy + 2] : (Real)1;
                const Real wZwY = wZ * wY;
                for (int ix = s0; ix < e0; ix++) {
                    const Real wX = wx ? ga[ix + 2] : (Real)1;
                    const Real v = lab_at(rt, phi, gphi, b, 2 * dx - ix, 2 * dy - iy, 2 * dz - iz);
                    result = result + v * (wZwY * wX);
                }
            }
        }
        const double a = fabs((double)result);
        mx = a > mx ? a : mx;
    }
    __shared__ double red[512];
    red[t] = mx;
    __syncthreads();
    for (int s = 256; s > 0; s >>= 1) {
        if (t < s) red[t] = red[t] > red[t + s] ? red[t] : red[t + s];
        __syncthreads();
    }
    if (t == 0) detail[b] = red[0];
}

// New block i of a remap: kind 0 = copy of old block src[8i]; kind 1 = child
// src[8i+1] (x + 2y + 4z) of old block src[8i], by Hs prediction
// (BlockSplitter::_splitBlocks, source/MRAGcore/MRAGBlockSplitter.h:24-100):
// fine point d takes parent lab points s with 2s - d in {-1, 0, 1}, weights
// Hs = {1/2, 1, 1/2}, summed from 0 in (sz, sy, sx) ascending order; kind 2 =
// collapse of the 8 old blocks src[8i..8i+7] (child x + 2y + 4z) by Ha = {1}
// decimation (BlockCollapser::_filter, MRAGBlockCollapser.h:19-44), i.e. the
// child's cell at even coordinates.
template <typename Real>
__global__ void k_amr_remap(int nbn, RegionTable rt, const int *__restrict__ kind, const int *__restrict__ src,
                            const Real *__restrict__ f_old, const Real *__restrict__ g_old,
                            Real *__restrict__ f_new) {
    const long total = (long)nbn * BC;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int b = (int)(i / BC), c = (int)(i % BC);
        const int x = c % BS, y = (c / BS) % BS, z = c / (BS * BS);
        const int k = kind[b];
        const int *sr = src + 8 * (size_t)b;
        Real v = 0;
        if (k == 0) {
            v = f_old[(size_t)sr[0] * BC + c];
        } else if (k == 1) {
            const int p = sr[0], ch = sr[1];
            const int d[3] = {(ch & 1) * BS + x, ((ch >> 1) & 1) * BS + y, ((ch >> 2) & 1) * BS + z};
            int lo[3], n[3];
            double w[3][2];
            for (int a = 0; a < 3; ++a) {
                if ((d[a] & 1) == 0) {
                    lo[a] = d[a] / 2; n[a] = 1; w[a][0] = 1.0;
                } else {
                    lo[a] = (d[a] - 1) / 2; n[a] = 2; w[a][0] = 0.5; w[a][1] = 0.5;
                }
            }
            Real acc = 0;
            for (int iz = 0; iz < n[2]; ++iz)
                for (int iy = 0; iy < n[1]; ++iy) {
                    const double wZwY = w[2][iz] * w[1][iy];
                    for (int ix = 0; ix < n[0]; ++ix) {
                        const Real val = lab_at(rt, f_old, g_old, p, lo[0] + ix, lo[1] + iy, lo[2] + iz);
                        acc = acc + val * (Real)(wZwY * w[0][ix]);
                    }
                }
            v = acc;
        } else {
            const int ch = (x / 8) + 2 * (y / 8) + 4 * (z / 8);
            const int sx = 2 * (x % 8), sy = 2 * (y % 8), sz = 2 * (z % 8);
            v = (Real)0 + f_old[(size_t)sr[ch] * BC + sx + BS * (sy + BS * sz)] * (Real)1.0;
        }
        f_new[i] = v;
    }
}

// Block cell values onto the finest uniform grid of gpd^3 cells
// (Glioma_HG_UQ::_dumpUQoutput, source/Glioma/Glioma_HG_UQ.cpp:309-372):
// cell (x, y, z) of a block with spacing h lands at floor(pos / hf), hf = 1/gpd,
// replicated r^3 times. reference_rules: r = 1 if h == hf, 2 if h == 2 hf,
// 3 if h == 3 hf, else 4 -- as the reference does, including its 4^3 for
// coarser blocks; otherwise r = h / hf exactly. Blocks finer than hf are
// sampled at their cells on the coarse grid points.
template <typename Real>
__global__ void k_amr_dump(int nb, const int *__restrict__ level, const int *__restrict__ bidx,
                           const Real *__restrict__ phi, int gpd, int reference_rules, double *__restrict__ out) {
    const long total = (long)nb * BC;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int b = (int)(i / BC), c = (int)(i % BC);
        const int x = c % BS, y = (c / BS) % BS, z = c / (BS * BS);
        const long cells_at_level = (long)BS << level[b];  // cells per side at this level
        const long g[3] = {(long)bidx[3 * b] * BS + x, (long)bidx[3 * b + 1] * BS + y, (long)bidx[3 * b + 2] * BS + z};
        long m[3];
        int r;
        if (cells_at_level >= gpd) {
            const long ratio = cells_at_level / gpd;  // block cells per dump cell
            if ((g[0] % ratio) || (g[1] % ratio) || (g[2] % ratio)) continue;
            for (int a = 0; a < 3; ++a) m[a] = g[a] / ratio;
            r = 1;
        } else {
            const long ratio = gpd / cells_at_level;  // dump cells per block cell
            for (int a = 0; a < 3; ++a) m[a] = g[a] * ratio;
            r = (int)ratio;
            if (reference_rules) r = ratio == 1 ? 1 : (ratio == 2 ? 2 : (ratio == 3 ? 3 : 4));
        }
        const double v = (double)phi[i];
        for (int cz = 0; cz < r; ++cz)
            for (int cy = 0; cy < r; ++cy)
                for (int cx = 0; cx < r; ++cx) {
                    const long X = m[0] + cx, Y = m[1] + cy, Z = m[2] + cz;
                    if (X < gpd && Y < gpd && Z < gpd) out[X + gpd * (Y + (long)gpd * Z)] = v;
                }
    }
}

RegionTable region_table() {
    RegionTable rt;
    for (int c = 0; c < 27; ++c) rt.start[c] = region_start(c);
    return rt;
}

int grid_blocks(const Handle &h, long work) {
    const long blocks = (work + 255) / 256;
    const long cap = (long)h.num_sms * 8;
    return (int)(blocks < cap ? blocks : cap);
}

}  // namespace

int amr_region_start(int code) { return region_start(code); }

int amr_alloc(Handle &h) {
    const size_t sb = h.prec == GBG_PREC_F64 ? sizeof(double) : sizeof(float);
    const size_t cells = (size_t)h.amr.max_blocks * BC;
    const size_t ghosts = (size_t)h.amr.max_blocks * NG;
    void **bufs[] = {&h.amr.phi[0], &h.amr.phi[1], &h.amr.pw, &h.amr.pg, &h.amr.b0};
    for (void **b : bufs) GBG_CUDA_TRY(cudaMalloc(b, cells * sb));
    void **gb[] = {&h.amr.gphi, &h.amr.gpw, &h.amr.gpg};
    for (void **b : gb) GBG_CUDA_TRY(cudaMalloc(b, ghosts * sb));
    GBG_CUDA_TRY(cudaMalloc((void **)&h.amr.df, cells * 6 * sizeof(double)));
    GBG_CUDA_TRY(cudaMalloc((void **)&h.amr.level, (size_t)h.amr.max_blocks * sizeof(int)));
    GBG_CUDA_TRY(cudaMalloc((void **)&h.amr.gstart, (ghosts + 1) * sizeof(long)));
    if (h.prec == GBG_PREC_F32) GBG_CUDA_TRY(cudaMalloc((void **)&h.amr.gstart32, (ghosts + 1) * sizeof(int)));
    GBG_CUDA_TRY(cudaMalloc((void **)&h.amr.detail, (size_t)h.amr.max_blocks * sizeof(double)));
    GBG_CUDA_TRY(cudaMalloc(&h.amr.pw2, cells * sb));
    GBG_CUDA_TRY(cudaMalloc(&h.amr.pg2, cells * sb));
    GBG_CUDA_TRY(cudaMalloc((void **)&h.amr.bidx, (size_t)h.amr.max_blocks * 3 * sizeof(int)));
    GBG_CUDA_TRY(cudaMalloc((void **)&h.amr.rkind, (size_t)h.amr.max_blocks * sizeof(int)));
    GBG_CUDA_TRY(cudaMalloc((void **)&h.amr.rsrc, (size_t)h.amr.max_blocks * 8 * sizeof(int)));
    return GBG_OK;
}

void amr_free(Handle &h) {
    void *p[] = {h.amr.phi[0], h.amr.phi[1], h.amr.pw, h.amr.pg, h.amr.b0, h.amr.gphi, h.amr.gpw, h.amr.gpg,
                 h.amr.df, h.amr.level, h.amr.gstart, h.amr.gsrc_block, h.amr.gsrc_cell, h.amr.gw,
                 h.amr.gstart32, h.amr.gsrc32, h.amr.gw32,
                 h.amr.detail, h.amr.pw2, h.amr.pg2, h.amr.bidx, h.amr.rkind, h.amr.rsrc};
    for (void *q : p)
        if (q) cudaFree(q);
}

int amr_set_grid(Handle &h, int nb, const gbg_block *blocks, const double *pw, const double *pg,
                 const double *phi) {
    const size_t n = (size_t)nb * BC;
    std::vector<int> lv(nb), bi(3 * (size_t)nb);
    for (int i = 0; i < nb; ++i) {
        lv[i] = blocks[i].level;
        bi[3 * i] = blocks[i].ix;
        bi[3 * i + 1] = blocks[i].iy;
        bi[3 * i + 2] = blocks[i].iz;
    }
    GBG_CUDA_TRY(cudaMemcpyAsync(h.amr.level, lv.data(), nb * sizeof(int), cudaMemcpyHostToDevice, h.stream));
    GBG_CUDA_TRY(cudaMemcpyAsync(h.amr.bidx, bi.data(), bi.size() * sizeof(int), cudaMemcpyHostToDevice, h.stream));
    const double *src[3] = {pw, pg, phi};
    void *dst[3] = {h.amr.pw, h.amr.pg, h.amr.phi[0]};
    if (h.prec == GBG_PREC_F64) {
        for (int k = 0; k < 3; ++k)
            GBG_CUDA_TRY(cudaMemcpyAsync(dst[k], src[k], n * sizeof(double), cudaMemcpyHostToDevice, h.stream));
        GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    } else {
        std::vector<float> tmp(n);
        for (int k = 0; k < 3; ++k) {
            for (size_t i = 0; i < n; ++i) tmp[i] = (float)src[k][i];
            GBG_CUDA_TRY(cudaMemcpy(dst[k], tmp.data(), n * sizeof(float), cudaMemcpyHostToDevice));
        }
    }
    h.amr.nb = nb;
    h.amr.cur = 0;
    h.amr.hblocks.assign(blocks, blocks + nb);
    h.amr.ghosts_valid = false;
    h.amr.tables_valid = false;
    return GBG_OK;
}

int amr_set_ghosts(Handle &h, const long *start, const int *src_block, const int *src_cell, const double *w,
                   long nentries) {
    const long ng = (long)h.amr.nb * NG;
    for (long i = 0; i < ng; ++i)
        if (start[i + 1] < start[i]) {
            set_error("ghost table start offsets must not decrease");
            return GBG_ERR_ARG;
        }
    if (start[0] != 0 || start[ng] != nentries) {
        set_error("ghost table start offsets must span [0, nentries]");
        return GBG_ERR_ARG;
    }
    for (long k = 0; k < nentries; ++k)
        if (src_block[k] < 0 || src_block[k] >= h.amr.nb || src_cell[k] < 0 || src_cell[k] >= BC) {
            set_error("ghost table entry points outside the grid");
            return GBG_ERR_ARG;
        }
    if (h.prec == GBG_PREC_F32 && nentries > 0x7fffffffL) {
        set_error("ghost tables too large for the fast mode (2^31 entries)");
        return GBG_ERR_ARG;
    }
    if (h.amr.gsrc_block) cudaFree(h.amr.gsrc_block);
    if (h.amr.gsrc_cell) cudaFree(h.amr.gsrc_cell);
    if (h.amr.gw) cudaFree(h.amr.gw);
    if (h.amr.gsrc32) cudaFree(h.amr.gsrc32);
    if (h.amr.gw32) cudaFree(h.amr.gw32);
    h.amr.gsrc_block = nullptr;
    h.amr.gsrc_cell = nullptr;
    h.amr.gw = nullptr;
    h.amr.gsrc32 = nullptr;
    h.amr.gw32 = nullptr;
    const size_t ne = nentries > 0 ? (size_t)nentries : 1;
    GBG_CUDA_TRY(cudaMalloc((void **)&h.amr.gsrc_block, ne * sizeof(int)));
    GBG_CUDA_TRY(cudaMalloc((void **)&h.amr.gsrc_cell, ne * sizeof(int)));
    GBG_CUDA_TRY(cudaMalloc((void **)&h.amr.gw, ne * sizeof(double)));
    GBG_CUDA_TRY(cudaMemcpy(h.amr.gstart, start, (ng + 1) * sizeof(long), cudaMemcpyHostToDevice));
    if (nentries > 0) {
        GBG_CUDA_TRY(cudaMemcpy(h.amr.gsrc_block, src_block, nentries * sizeof(int), cudaMemcpyHostToDevice));
        GBG_CUDA_TRY(cudaMemcpy(h.amr.gsrc_cell, src_cell, nentries * sizeof(int), cudaMemcpyHostToDevice));
        GBG_CUDA_TRY(cudaMemcpy(h.amr.gw, w, nentries * sizeof(double), cudaMemcpyHostToDevice));
    }
    if (h.prec == GBG_PREC_F32) {
        GBG_CUDA_TRY(cudaMalloc((void **)&h.amr.gsrc32, ne * sizeof(int)));
        GBG_CUDA_TRY(cudaMalloc((void **)&h.amr.gw32, ne * sizeof(float)));
        k_compact_tables<<<grid_blocks(h, std::max(ng + 1, nentries)), 256, 0, h.stream>>>(
            ng, nentries, h.amr.gstart, h.amr.gsrc_block, h.amr.gsrc_cell, h.amr.gw, h.amr.gstart32, h.amr.gsrc32,
            h.amr.gw32);
        h.launches++;
    }
    // the anatomy's ghosts are static between regrids
    const int g = grid_blocks(h, ng);
    if (h.prec == GBG_PREC_F64) {
        k_ghost_eval<double><<<g, 256, 0, h.stream>>>(h.amr.nb, h.amr.gstart, h.amr.gsrc_block, h.amr.gsrc_cell,
                                                      h.amr.gw, (const double *)h.amr.pw, (double *)h.amr.gpw);
        k_ghost_eval<double><<<g, 256, 0, h.stream>>>(h.amr.nb, h.amr.gstart, h.amr.gsrc_block, h.amr.gsrc_cell,
                                                      h.amr.gw, (const double *)h.amr.pg, (double *)h.amr.gpg);
    } else {
        k_ghost_eval<float><<<g, 256, 0, h.stream>>>(h.amr.nb, h.amr.gstart, h.amr.gsrc_block, h.amr.gsrc_cell,
                                                     h.amr.gw, (const float *)h.amr.pw, (float *)h.amr.gpw);
        k_ghost_eval<float><<<g, 256, 0, h.stream>>>(h.amr.nb, h.amr.gstart, h.amr.gsrc_block, h.amr.gsrc_cell,
                                                     h.amr.gw, (const float *)h.amr.pg, (float *)h.amr.gpg);
    }
    h.launches += 2;
    GBG_CUDA_TRY(cudaGetLastError());
    h.amr.ghosts_valid = true;
    h.amr.tables_valid = false;
    return GBG_OK;
}

int amr_steps(Handle &h, double Dw, double Dg, double rho, double dt, long nsteps) {
    if (!h.amr.ghosts_valid) {
        set_error("ghost tables not set");
        return GBG_ERR_STATE;
    }
    const RegionTable rt = region_table();
    const long cells = (long)h.amr.nb * BC, ng = (long)h.amr.nb * NG;
    const int gc = grid_blocks(h, cells), gg = grid_blocks(h, ng);
    const bool f64 = h.prec == GBG_PREC_F64;
    if (h.prec == GBG_PREC_F32) {
        // fast mode: unit coefficients for the ratio Dg/Dw (rounded to float, as
        // the uniform fast path does), the 7-float table in the df storage
        float *tab = reinterpret_cast<float *>(h.amr.df);
        const bool fused = h.amr.fast_variant == 0;
        // fused form: per-face tables in the same storage
        float *fx = tab, *fy = tab + (size_t)h.amr.nb * NFX, *fz = tab + 2 * (size_t)h.amr.nb * NFX;
        unsigned char *msk = reinterpret_cast<unsigned char *>(tab + 3 * (size_t)h.amr.nb * NFX);
        if (!h.amr.tables_valid || h.amr.tab_Dw != Dw || h.amr.tab_Dg != Dg) {
            if (fused)
                k_amr_fast_faces<<<grid_blocks(h, (long)h.amr.nb * (3L * NFX + BC)), 256, 0, h.stream>>>(
                    h.amr.nb, rt, (const float *)h.amr.pw, (const float *)h.amr.pg, (const float *)h.amr.gpw,
                    (const float *)h.amr.gpg, (double)(float)(Dg / Dw), fx, fy, fz, msk);
            else
                k_amr_fast_tables<<<gc, 256, 0, h.stream>>>(h.amr.nb, rt, (const float *)h.amr.pw,
                                                            (const float *)h.amr.pg, (const float *)h.amr.gpw,
                                                            (const float *)h.amr.gpg, (double)(float)(Dg / Dw),
                                                            tab);
            h.launches++;
            h.amr.tab_Dw = Dw;
            h.amr.tab_Dg = Dg;
            h.amr.tables_valid = true;
        }
        const int gb = std::min(h.amr.nb, h.num_sms * 8);
        if (fused) {
            for (long s = 0; s < nsteps; ++s) {
                void *in = h.amr.phi[h.amr.cur], *out = h.amr.phi[h.amr.cur ^ 1];
                k_amr_fast_step_fused<<<gb, 256, 0, h.stream>>>(h.amr.nb, rt, h.amr.level, (const float *)in,
                                                                h.amr.gstart32, h.amr.gsrc32, h.amr.gw32, fx, fy, fz,
                                                                msk, (float *)out, Dw, rho, dt);
                h.launches++;
                h.amr.cur ^= 1;
            }
            GBG_CUDA_TRY(cudaGetLastError());
            return GBG_OK;
        }
        for (long s = 0; s < nsteps; ++s) {
            void *in = h.amr.phi[h.amr.cur], *out = h.amr.phi[h.amr.cur ^ 1];
            k_ghost_eval<float><<<gg, 256, 0, h.stream>>>(h.amr.nb, h.amr.gstart, h.amr.gsrc_block, h.amr.gsrc_cell,
                                                          h.amr.gw, (const float *)in, (float *)h.amr.gphi);
            k_amr_fast_step<<<gb, 256, 0, h.stream>>>(h.amr.nb, rt, h.amr.level, (const float *)in,
                                                      (const float *)h.amr.gphi, tab, (float *)out, Dw, rho, dt);
            h.launches += 2;
            h.amr.cur ^= 1;
        }
        GBG_CUDA_TRY(cudaGetLastError());
        return GBG_OK;
    }
    if (!h.amr.tables_valid || h.amr.tab_Dw != Dw || h.amr.tab_Dg != Dg) {
        if (f64)
            k_amr_tables<double><<<gc, 256, 0, h.stream>>>(h.amr.nb, rt, (const double *)h.amr.pw,
                                                           (const double *)h.amr.pg, (const double *)h.amr.gpw,
                                                           (const double *)h.amr.gpg, Dw, Dg,
                                                           (double *)h.amr.b0, h.amr.df);
        else
            k_amr_tables<float><<<gc, 256, 0, h.stream>>>(h.amr.nb, rt, (const float *)h.amr.pw,
                                                          (const float *)h.amr.pg, (const float *)h.amr.gpw,
                                                          (const float *)h.amr.gpg, (float)Dw, (float)Dg,
                                                          (float *)h.amr.b0, h.amr.df);
        h.launches++;
        h.amr.tab_Dw = Dw;
        h.amr.tab_Dg = Dg;
        h.amr.tables_valid = true;
    }
    for (long s = 0; s < nsteps; ++s) {
        void *in = h.amr.phi[h.amr.cur], *out = h.amr.phi[h.amr.cur ^ 1];
        if (f64) {
            k_ghost_eval<double><<<gg, 256, 0, h.stream>>>(h.amr.nb, h.amr.gstart, h.amr.gsrc_block,
                                                           h.amr.gsrc_cell, h.amr.gw, (const double *)in,
                                                           (double *)h.amr.gphi);
            k_amr_step<double><<<gc, 256, 0, h.stream>>>(h.amr.nb, rt, h.amr.level, (const double *)in,
                                                         (const double *)h.amr.gphi, (const double *)h.amr.b0,
                                                         h.amr.df, (double *)out, rho, dt);
        } else {
            k_ghost_eval<float><<<gg, 256, 0, h.stream>>>(h.amr.nb, h.amr.gstart, h.amr.gsrc_block,
                                                          h.amr.gsrc_cell, h.amr.gw, (const float *)in,
                                                          (float *)h.amr.gphi);
            k_amr_step<float><<<gc, 256, 0, h.stream>>>(h.amr.nb, rt, h.amr.level, (const float *)in,
                                                        (const float *)h.amr.gphi, (const float *)h.amr.b0,
                                                        h.amr.df, (float *)out, (float)rho, dt);
        }
        h.launches += 2;
        h.amr.cur ^= 1;
    }
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
}

int amr_get_phi(Handle &h, double *phi) {
    const size_t n = (size_t)h.amr.nb * BC;
    if (h.prec == GBG_PREC_F64) {
        GBG_CUDA_TRY(cudaMemcpyAsync(phi, h.amr.phi[h.amr.cur], n * sizeof(double), cudaMemcpyDeviceToHost, h.stream));
        GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    } else {
        std::vector<float> tmp(n);
        GBG_CUDA_TRY(cudaMemcpyAsync(tmp.data(), h.amr.phi[h.amr.cur], n * sizeof(float), cudaMemcpyDeviceToHost,
                                     h.stream));
        GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
        for (size_t i = 0; i < n; ++i) phi[i] = tmp[i];
    }
    return GBG_OK;
}

int amr_fwt_detail(Handle &h, double *detail) {
    if (!h.amr.ghosts_valid) {
        set_error("ghost tables not set");
        return GBG_ERR_STATE;
    }
    const RegionTable rt = region_table();
    const long ng = (long)h.amr.nb * NG;
    const int gg = grid_blocks(h, ng);
    void *in = h.amr.phi[h.amr.cur];
    if (h.prec == GBG_PREC_F64) {
        k_ghost_eval<double><<<gg, 256, 0, h.stream>>>(h.amr.nb, h.amr.gstart, h.amr.gsrc_block, h.amr.gsrc_cell,
                                                       h.amr.gw, (const double *)in, (double *)h.amr.gphi);
        k_amr_fwt<double><<<h.amr.nb, 512, 0, h.stream>>>(h.amr.nb, rt, (const double *)in,
                                                          (const double *)h.amr.gphi, h.amr.detail);
    } else {
        k_ghost_eval<float><<<gg, 256, 0, h.stream>>>(h.amr.nb, h.amr.gstart, h.amr.gsrc_block, h.amr.gsrc_cell,
                                                      h.amr.gw, (const float *)in, (float *)h.amr.gphi);
        k_amr_fwt<float><<<h.amr.nb, 512, 0, h.stream>>>(h.amr.nb, rt, (const float *)in,
                                                         (const float *)h.amr.gphi, h.amr.detail);
    }
    h.launches += 2;
    GBG_CUDA_TRY(cudaGetLastError());
    GBG_CUDA_TRY(cudaMemcpyAsync(detail, h.amr.detail, h.amr.nb * sizeof(double), cudaMemcpyDeviceToHost, h.stream));
    GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    return GBG_OK;
}

int amr_remap(Handle &h, int nbn, const gbg_block *blocks, const int *kind, const int *src) {
    if (!h.amr.ghosts_valid) {
        set_error("the remap reads the current grid's ghosts: set its ghost tables first");
        return GBG_ERR_STATE;
    }
    std::vector<int> lv(nbn), bi(3 * (size_t)nbn);
    for (int i = 0; i < nbn; ++i) {
        lv[i] = blocks[i].level;
        bi[3 * i] = blocks[i].ix;
        bi[3 * i + 1] = blocks[i].iy;
        bi[3 * i + 2] = blocks[i].iz;
    }
    const RegionTable rt = region_table();
    const long ng = (long)h.amr.nb * NG, cells = (long)nbn * BC;
    const int gg = grid_blocks(h, ng), gc = grid_blocks(h, cells);
    GBG_CUDA_TRY(cudaMemcpyAsync(h.amr.rkind, kind, nbn * sizeof(int), cudaMemcpyHostToDevice, h.stream));
    GBG_CUDA_TRY(cudaMemcpyAsync(h.amr.rsrc, src, 8 * (size_t)nbn * sizeof(int), cudaMemcpyHostToDevice, h.stream));
    void *pin = h.amr.phi[h.amr.cur], *pout = h.amr.phi[h.amr.cur ^ 1];
    if (h.prec == GBG_PREC_F64) {
        k_ghost_eval<double><<<gg, 256, 0, h.stream>>>(h.amr.nb, h.amr.gstart, h.amr.gsrc_block, h.amr.gsrc_cell,
                                                       h.amr.gw, (const double *)pin, (double *)h.amr.gphi);
        k_amr_remap<double><<<gc, 256, 0, h.stream>>>(nbn, rt, h.amr.rkind, h.amr.rsrc, (const double *)pin,
                                                      (const double *)h.amr.gphi, (double *)pout);
        k_amr_remap<double><<<gc, 256, 0, h.stream>>>(nbn, rt, h.amr.rkind, h.amr.rsrc, (const double *)h.amr.pw,
                                                      (const double *)h.amr.gpw, (double *)h.amr.pw2);
        k_amr_remap<double><<<gc, 256, 0, h.stream>>>(nbn, rt, h.amr.rkind, h.amr.rsrc, (const double *)h.amr.pg,
                                                      (const double *)h.amr.gpg, (double *)h.amr.pg2);
    } else {
        k_ghost_eval<float><<<gg, 256, 0, h.stream>>>(h.amr.nb, h.amr.gstart, h.amr.gsrc_block, h.amr.gsrc_cell,
                                                      h.amr.gw, (const float *)pin, (float *)h.amr.gphi);
        k_amr_remap<float><<<gc, 256, 0, h.stream>>>(nbn, rt, h.amr.rkind, h.amr.rsrc, (const float *)pin,
                                                     (const float *)h.amr.gphi, (float *)pout);
        k_amr_remap<float><<<gc, 256, 0, h.stream>>>(nbn, rt, h.amr.rkind, h.amr.rsrc, (const float *)h.amr.pw,
                                                     (const float *)h.amr.gpw, (float *)h.amr.pw2);
        k_amr_remap<float><<<gc, 256, 0, h.stream>>>(nbn, rt, h.amr.rkind, h.amr.rsrc, (const float *)h.amr.pg,
                                                     (const float *)h.amr.gpg, (float *)h.amr.pg2);
    }
    h.launches += 4;
    GBG_CUDA_TRY(cudaGetLastError());
    GBG_CUDA_TRY(cudaMemcpyAsync(h.amr.level, lv.data(), nbn * sizeof(int), cudaMemcpyHostToDevice, h.stream));
    GBG_CUDA_TRY(cudaMemcpyAsync(h.amr.bidx, bi.data(), bi.size() * sizeof(int), cudaMemcpyHostToDevice, h.stream));
    GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    std::swap(h.amr.pw, h.amr.pw2);
    std::swap(h.amr.pg, h.amr.pg2);
    h.amr.cur ^= 1;
    h.amr.nb = nbn;
    h.amr.hblocks.assign(blocks, blocks + nbn);
    h.amr.ghosts_valid = false;
    h.amr.tables_valid = false;
    return GBG_OK;
}

int amr_dump_uniform(Handle &h, int gpd, int reference_rules, double *out) {
    const size_t n3 = (size_t)gpd * gpd * gpd;
    double *d = nullptr;
    GBG_CUDA_TRY(cudaMalloc((void **)&d, n3 * sizeof(double)));
    cudaError_t e = cudaMemsetAsync(d, 0, n3 * sizeof(double), h.stream);
    const long cells = (long)h.amr.nb * BC;
    if (e == cudaSuccess) {
        if (h.prec == GBG_PREC_F64)
            k_amr_dump<double><<<grid_blocks(h, cells), 256, 0, h.stream>>>(
                h.amr.nb, h.amr.level, h.amr.bidx, (const double *)h.amr.phi[h.amr.cur], gpd, reference_rules, d);
        else
            k_amr_dump<float><<<grid_blocks(h, cells), 256, 0, h.stream>>>(
                h.amr.nb, h.amr.level, h.amr.bidx, (const float *)h.amr.phi[h.amr.cur], gpd, reference_rules, d);
        h.launches++;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, n3 * sizeof(double), cudaMemcpyDeviceToHost, h.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h.stream);
    cudaFree(d);
    if (e != cudaSuccess) {
        set_error(std::string("amr dump: ") + cudaGetErrorString(e));
        return GBG_ERR_CUDA;
    }
    return GBG_OK;
}

}  // namespace gbg
