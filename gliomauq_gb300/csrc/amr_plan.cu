// Adaptive block grid, host side: the ghost instruction tables of any
// periodic block tree, MRAG's refinement and compression plans, the
// automatic regrids of the Glioma time loop, and that loop.
//
// Ghost tables (what MRAG_BBInfoCreator builds, source/MRAGcore/MRAG_BBInfoCreator.inl:902-1316,
// with Grid::_computeBoundaryInfo, MRAGrid.inl:514-700): a ghost of block b at
// lab coordinate g (stencil [-1, 2), BlockLab::load order) is the point
// p = 16 * index(b) + g on b's level (periodic). A point p on level l is
// expanded depth first:
//   * the leaf containing its position is on level l: one term, that cell;
//   * the leaf is finer (interpolating wavelets are node-centred, so p is the
//     point 2p of level l + 1): the expansion of 2p on level l + 1 (analysis
//     with Ha = {1});
//   * the leaf is coarser: sum over j of Hs(2j - p) times the expansion of j
//     on level l - 1 (synthesis with Hs = {1/2, 1, 1/2}: one coarse point for
//     even p, the two neighbours with weight 1/2 for odd p), j visited z, y,
//     x outermost first as MRAG's request matrices are.
// The weights of a term are the per-axis products along its path; all are
// powers of two, so their product is exact in any floating type. Same-level
// ghosts (most of them) are single copies.
//
// Neighbourhood (Grid::_computeNeighborhood, MRAGrid.inl:841-1150): block B,
// or one of its periodic images (B shifted by one domain length along any
// subset of the axes), is a neighbour of A when its extent touches or overlaps
// A's; images are MRAG's ghost nodes.
//
// Refinement plan (Refiner_SpaceExtension::createPlan,
// source/MRAGscience/MRAGRefiner_SpaceExtension.h:25-67, then
// Refiner::createPlan, source/MRAGcore/MRAGRefiner.h:45-195): the flagged
// blocks, plus every block with a finer neighbour that is not an image, minus
// the blocks on the maximum level; then, until nothing changes, every
// neighbour (images included) more than one level coarser than the children
// of a block to refine is refined too. Each refined block becomes its eight
// children (BlockSplitter prediction on the device).
//
// Compression plan (Compressor::createPlan, source/MRAGcore/MRAGCompressor.h:68-144):
// eight sibling blocks collapse into their parent when all are flagged and
// every neighbour of every one of them (images included) is within one level
// of the parent (BlockCollapser decimation on the device).
//
// Automatic regrids (Science::AutomaticRefinement / AutomaticCompression,
// source/MRAGscience/MRAGScienceCore.h:42-177) compare the per-block detail of
// BlockFWT with the tolerances; the compression repeats until a pass
// collapses nothing, and a block that was not flagged in an earlier pass of
// the same call is not examined again.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstring>
#include <set>
#include <thread>
#include <tuple>
#include <vector>

#include "gbg_internal.cuh"

namespace gbg {
namespace {

constexpr int BS = 16;
constexpr int NG = 1736;

struct Term {
    int block, cell;
    double w;
};

// Leaves of a block tree with lookup by level and index.
class Tree {
  public:
    std::vector<gbg_block> b;
    int maxl = 0;
    std::vector<std::vector<int>> at;  // at[L][(iz * m + iy) * m + ix] -> leaf or -1

    int build(const gbg_block *blocks, int nb) {
        b.assign(blocks, blocks + nb);
        maxl = 0;
        for (const gbg_block &x : b) {
            if (x.level < 0 || x.level > 10) return GBG_ERR_ARG;
            maxl = std::max(maxl, x.level);
        }
        at.assign(maxl + 1, {});
        for (int L = 0; L <= maxl; ++L) at[L].assign((size_t)1 << (3 * L), -1);
        for (int i = 0; i < nb; ++i) {
            const gbg_block &x = b[i];
            const int m = 1 << x.level;
            if (x.ix < 0 || x.iy < 0 || x.iz < 0 || x.ix >= m || x.iy >= m || x.iz >= m) return GBG_ERR_ARG;
            int &slot = at[x.level][((size_t)x.iz * m + x.iy) * m + x.ix];
            if (slot >= 0) return GBG_ERR_ARG;
            slot = i;
        }
        // the leaves must tile the unit cube: as many finest-level units as
        // the cube has, and no leaf inside another
        const long U = 1L << maxl;
        long covered = 0;
        for (const gbg_block &x : b) covered += 1L << (3 * (maxl - x.level));
        if (covered != U * U * U) return GBG_ERR_ARG;
        for (const gbg_block &x : b)
            for (int L = 0; L < x.level; ++L) {
                const int sh = x.level - L;
                if (leaf(L, x.ix >> sh, x.iy >> sh, x.iz >> sh) >= 0) return GBG_ERR_ARG;
            }
        return GBG_OK;
    }

    int leaf(int L, long ix, long iy, long iz) const {
        const long m = 1L << L;
        if (ix < 0 || iy < 0 || iz < 0 || ix >= m || iy >= m || iz >= m) return -1;
        return at[L][((size_t)iz * m + iy) * m + ix];
    }

    // leaf whose extent contains the position of point p (wrapped) of level l
    int leaf_of_point(int l, const long p[3]) const {
        for (int L = 0; L <= maxl; ++L) {
            long q[3];
            for (int a = 0; a < 3; ++a) q[a] = L >= l ? (p[a] << (L - l)) >> 4 : p[a] >> (l - L + 4);
            const int s = leaf(L, q[0], q[1], q[2]);
            if (s >= 0) return s;
        }
        return -1;
    }

    // depth-first expansion of point p of level l (see the file comment)
    bool expand(int l, long p0, long p1, long p2, double wx, double wy, double wz, std::vector<Term> &out,
                int depth = 0) const {
        if (depth > 64 || l < 0 || l > maxl) return false;
        const long M = (long)BS << l;
        const long p[3] = {((p0 % M) + M) % M, ((p1 % M) + M) % M, ((p2 % M) + M) % M};
        const int s = leaf_of_point(l, p);
        if (s < 0) return false;
        const gbg_block &x = b[s];
        if (x.level == l) {
            const int cx = (int)(p[0] - (long)x.ix * BS), cy = (int)(p[1] - (long)x.iy * BS),
                      cz = (int)(p[2] - (long)x.iz * BS);
            out.push_back({s, cx + BS * (cy + BS * cz), wx * wy * wz});
            return true;
        }
        if (x.level > l) return expand(l + 1, 2 * p[0], 2 * p[1], 2 * p[2], wx, wy, wz, out, depth + 1);
        long j0[3], nj[3];
        for (int a = 0; a < 3; ++a) {
            if ((p[a] & 1) == 0) {
                j0[a] = p[a] / 2;
                nj[a] = 1;
            } else {
                j0[a] = (p[a] - 1) / 2;
                nj[a] = 2;
            }
        }
        for (long kz = 0; kz < nj[2]; ++kz) {
            const double az = nj[2] == 1 ? 1.0 : 0.5;
            for (long ky = 0; ky < nj[1]; ++ky) {
                const double ay = nj[1] == 1 ? 1.0 : 0.5;
                for (long kx = 0; kx < nj[0]; ++kx) {
                    const double ax = nj[0] == 1 ? 1.0 : 0.5;
                    if (!expand(l - 1, j0[0] + kx, j0[1] + ky, j0[2] + kz, wx * ax, wy * ay, wz * az, out,
                                depth + 1))
                        return false;
                }
            }
        }
        return true;
    }

    // neighbours of leaf a: (leaf, image) pairs, image = whether the touching
    // copy is a periodic image (shift != 0); one entry per (leaf, shift)
    void neighbours(int a, std::vector<std::pair<int, bool>> &out) const {
        out.clear();
        const gbg_block &x = b[a];
        const long U = 1L << maxl, s = 1L << (maxl - x.level);
        const long lo[3] = {(long)x.ix * s, (long)x.iy * s, (long)x.iz * s};
        std::set<std::tuple<int, int, int, int>> seen;  // (leaf, shift x, y, z)
        for (long uz = lo[2] - 1; uz <= lo[2] + s; ++uz)
            for (long uy = lo[1] - 1; uy <= lo[1] + s; ++uy)
                for (long ux = lo[0] - 1; ux <= lo[0] + s; ++ux) {
                    const bool inside = ux >= lo[0] && ux < lo[0] + s && uy >= lo[1] && uy < lo[1] + s &&
                                        uz >= lo[2] && uz < lo[2] + s;
                    if (inside) continue;
                    const long w[3] = {((ux % U) + U) % U, ((uy % U) + U) % U, ((uz % U) + U) % U};
                    const int sh[3] = {(int)((ux - w[0]) / U), (int)((uy - w[1]) / U), (int)((uz - w[2]) / U)};
                    const long p[3] = {w[0] * BS, w[1] * BS, w[2] * BS};  // a point of that unit
                    const int n = leaf_of_point(maxl, p);
                    if (n < 0) continue;
                    const bool image = sh[0] || sh[1] || sh[2];
                    if (n == a && !image) continue;
                    if (seen.insert(std::make_tuple(n, sh[0], sh[1], sh[2])).second) out.push_back({n, image});
                }
    }
};

// lab coordinates of the 1736 ghosts in BlockLab::load order
void ghost_coords(std::vector<std::array<int, 3>> &g) {
    g.clear();
    for (int code = 0; code < 27; ++code) {
        if (code == 13) continue;
        const int d[3] = {code % 3 - 1, (code / 3) % 3 - 1, (code / 9) % 3 - 1};
        int lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
            lo[a] = d[a] < 0 ? -1 : (d[a] == 0 ? 0 : BS);
            hi[a] = d[a] == 0 ? BS : lo[a] + 1;
        }
        for (int z = lo[2]; z < hi[2]; ++z)
            for (int y = lo[1]; y < hi[1]; ++y)
                for (int x = lo[0]; x < hi[0]; ++x) g.push_back({x, y, z});
    }
}

struct Tables {
    std::vector<long> start;
    std::vector<int> src_block, src_cell;
    std::vector<double> w;
};

int compile_tables(const Tree &t, Tables &out) {
    std::vector<std::array<int, 3>> g;
    ghost_coords(g);
    const int nb = (int)t.b.size();
    // per block: its terms, and the term count of each of its ghosts
    std::vector<std::vector<Term>> terms(nb);
    std::vector<std::vector<int>> counts(nb);
    std::vector<int> bad(nb, 0);
    auto work = [&](int b0, int b1) {
        for (int i = b0; i < b1; ++i) {
            std::vector<Term> &o = terms[i];
            std::vector<int> &c = counts[i];
            o.reserve(NG + 256);
            c.resize(NG);
            const gbg_block &x = t.b[i];
            for (int k = 0; k < NG; ++k) {
                const size_t before = o.size();
                if (!t.expand(x.level, (long)x.ix * BS + g[k][0], (long)x.iy * BS + g[k][1],
                              (long)x.iz * BS + g[k][2], 1.0, 1.0, 1.0, o)) {
                    bad[i] = 1;
                    return;
                }
                c[k] = (int)(o.size() - before);
            }
        }
    };
    unsigned nt = std::thread::hardware_concurrency();
    nt = std::max(1u, std::min(nt, 16u));
    if (nb < 64) nt = 1;
    std::vector<std::thread> th;
    for (unsigned k = 0; k < nt; ++k) {
        const int b0 = (int)((long)nb * k / nt), b1 = (int)((long)nb * (k + 1) / nt);
        th.emplace_back(work, b0, b1);
    }
    for (std::thread &x : th) x.join();
    for (int i = 0; i < nb; ++i)
        if (bad[i]) {
            set_error("ghost expansion found no block: the blocks do not form a valid tree");
            return GBG_ERR_ARG;
        }
    size_t total = 0;
    for (int i = 0; i < nb; ++i) total += terms[i].size();
    out.start.assign((size_t)nb * NG + 1, 0);
    out.src_block.resize(total);
    out.src_cell.resize(total);
    out.w.resize(total);
    size_t e = 0, gi = 0;
    for (int i = 0; i < nb; ++i) {
        size_t k = 0;
        for (int q = 0; q < NG; ++q) {
            out.start[gi++] = (long)e;
            for (int r = 0; r < counts[i][q]; ++r, ++k, ++e) {
                out.src_block[e] = terms[i][k].block;
                out.src_cell[e] = terms[i][k].cell;
                out.w[e] = terms[i][k].w;
            }
        }
    }
    out.start[gi] = (long)e;
    return GBG_OK;
}

struct Plan {
    std::vector<gbg_block> blocks;
    std::vector<int> kind, src;  // src: 8 per new block
};

void keep(Plan &p, const gbg_block &x, int a) {
    p.blocks.push_back(x);
    p.kind.push_back(GBG_REMAP_COPY);
    for (int k = 0; k < 8; ++k) p.src.push_back(k == 0 ? a : 0);
}

// Refiner_SpaceExtension + Refiner::createPlan; returns the number of refined blocks
int plan_refine(const Tree &t, const std::vector<char> &flagged, int max_level, Plan &plan) {
    const int nb = (int)t.b.size();
    std::vector<char> victim(nb, 0);
    std::vector<std::vector<std::pair<int, bool>>> nbr(nb);
    for (int a = 0; a < nb; ++a) t.neighbours(a, nbr[a]);
    for (int a = 0; a < nb; ++a) {
        bool r = flagged[a] != 0;
        for (const auto &n : nbr[a])
            if (!n.second && t.b[n.first].level > t.b[a].level) {
                r = true;
                break;
            }
        if (max_level >= 0 && t.b[a].level >= max_level) r = false;
        victim[a] = r;
    }
    std::vector<int> frontier;
    for (int a = 0; a < nb; ++a)
        if (victim[a]) frontier.push_back(a);
    while (!frontier.empty()) {
        std::vector<int> next;
        for (int v : frontier) {
            const int child_level = t.b[v].level + 1;
            for (const auto &n : nbr[v])
                if (std::abs(t.b[n.first].level - child_level) > 1 && !victim[n.first]) {
                    victim[n.first] = 1;
                    next.push_back(n.first);
                }
        }
        frontier.swap(next);
    }
    plan.blocks.clear();
    plan.kind.clear();
    plan.src.clear();
    int refined = 0;
    for (int a = 0; a < nb; ++a) {
        const gbg_block &x = t.b[a];
        if (!victim[a]) {
            keep(plan, x, a);
            continue;
        }
        ++refined;
        for (int c = 0; c < 8; ++c) {
            plan.blocks.push_back({x.level + 1, 2 * x.ix + (c & 1), 2 * x.iy + ((c >> 1) & 1), 2 * x.iz + ((c >> 2) & 1)});
            plan.kind.push_back(GBG_REMAP_SPLIT);
            for (int k = 0; k < 8; ++k) plan.src.push_back(k == 0 ? a : (k == 1 ? c : 0));
        }
    }
    return refined;
}

// Compressor::createPlan; returns the number of collapses
int plan_compress(const Tree &t, const std::vector<char> &flagged, Plan &plan) {
    const int nb = (int)t.b.size();
    std::vector<int> collapse_of(nb, -1);  // leaf -> collapse group
    std::vector<std::array<int, 8>> groups;
    std::vector<gbg_block> parents;
    std::vector<std::pair<int, bool>> nbr;
    for (int a = 0; a < nb; ++a) {
        const gbg_block &x = t.b[a];
        if (x.level == 0 || collapse_of[a] >= 0) continue;
        if ((x.ix & 1) || (x.iy & 1) || (x.iz & 1)) continue;  // each family from its first child
        std::array<int, 8> ch;
        bool ok = true;
        for (int c = 0; c < 8 && ok; ++c) {
            ch[c] = t.leaf(x.level, x.ix + (c & 1), x.iy + ((c >> 1) & 1), x.iz + ((c >> 2) & 1));
            ok = ch[c] >= 0 && flagged[ch[c]];
        }
        if (!ok) continue;
        const int parent_level = x.level - 1;
        for (int c = 0; c < 8 && ok; ++c) {
            t.neighbours(ch[c], nbr);
            for (const auto &n : nbr)
                if (std::abs(t.b[n.first].level - parent_level) > 1) {
                    ok = false;
                    break;
                }
        }
        if (!ok) continue;
        for (int c = 0; c < 8; ++c) collapse_of[ch[c]] = (int)groups.size();
        groups.push_back(ch);
        parents.push_back({parent_level, x.ix / 2, x.iy / 2, x.iz / 2});
    }
    plan.blocks.clear();
    plan.kind.clear();
    plan.src.clear();
    for (int a = 0; a < nb; ++a)
        if (collapse_of[a] < 0) keep(plan, t.b[a], a);
    for (size_t gi = 0; gi < groups.size(); ++gi) {
        plan.blocks.push_back(parents[gi]);
        plan.kind.push_back(GBG_REMAP_COLLAPSE);
        for (int k = 0; k < 8; ++k) plan.src.push_back(groups[gi][k]);
    }
    return (int)groups.size();
}

// ---- device-handle drivers -----------------------------------------------------

int install_tables(Handle &h) {
    Tree t;
    if (t.build(h.amr.hblocks.data(), (int)h.amr.hblocks.size()) != GBG_OK) {
        set_error("the grid's blocks do not tile the unit cube as a block tree");
        return GBG_ERR_ARG;
    }
    Tables tb;
    if (int rc = compile_tables(t, tb)) return rc;
    return amr_set_ghosts(h, tb.start.data(), tb.src_block.data(), tb.src_cell.data(), tb.w.data(),
                          (long)tb.src_block.size());
}

int apply_plan(Handle &h, const Plan &p) {
    if ((int)p.blocks.size() > h.amr.max_blocks) {
        set_error("the regridded grid needs more blocks than the handle's max_blocks");
        return GBG_ERR_NOMEM;
    }
    if (int rc = amr_remap(h, (int)p.blocks.size(), p.blocks.data(), p.kind.data(), p.src.data())) return rc;
    return install_tables(h);
}

}  // namespace

int amr_build_ghosts(Handle &h) { return install_tables(h); }

int amr_auto_refine(Handle &h, double tol, int max_level, int *refined) {
    *refined = 0;
    const int nb = h.amr.nb;
    bool any = false;
    for (const gbg_block &x : h.amr.hblocks) any |= max_level < 0 || x.level < max_level;
    if (!any) return GBG_OK;
    std::vector<double> det(nb);
    if (int rc = amr_fwt_detail(h, det.data())) return rc;
    std::vector<char> flagged(nb, 0);
    bool some = false;
    for (int i = 0; i < nb; ++i) {
        const bool candidate = max_level < 0 || h.amr.hblocks[i].level < max_level;
        flagged[i] = candidate && det[i] >= tol;
        some |= flagged[i] != 0;
    }
    if (!some) return GBG_OK;
    Tree t;
    if (t.build(h.amr.hblocks.data(), nb) != GBG_OK) {
        set_error("the grid's blocks do not form a block tree");
        return GBG_ERR_ARG;
    }
    Plan p;
    *refined = plan_refine(t, flagged, max_level, p);
    return apply_plan(h, p);
}

int amr_auto_compress(Handle &h, double tol, int *collapsed) {
    *collapsed = 0;
    std::set<std::array<int, 4>> nice;
    while (true) {
        const int nb = h.amr.nb;
        std::vector<double> det(nb);
        std::vector<char> candidate(nb, 0), flagged(nb, 0);
        bool any = false;
        for (int i = 0; i < nb; ++i) {
            const gbg_block &x = h.amr.hblocks[i];
            candidate[i] = nice.count({x.level, x.ix, x.iy, x.iz}) == 0;
            any |= candidate[i] != 0;
        }
        if (!any) break;
        if (int rc = amr_fwt_detail(h, det.data())) return rc;
        bool some = false;
        for (int i = 0; i < nb; ++i) {
            if (!candidate[i]) continue;
            const gbg_block &x = h.amr.hblocks[i];
            if (det[i] < tol) {
                flagged[i] = 1;
                some = true;
            } else {
                nice.insert({x.level, x.ix, x.iy, x.iz});
            }
        }
        if (!some) break;
        Tree t;
        if (t.build(h.amr.hblocks.data(), nb) != GBG_OK) {
            set_error("the grid's blocks do not form a block tree");
            return GBG_ERR_ARG;
        }
        Plan p;
        const int n = plan_compress(t, flagged, p);
        if (n == 0) break;
        if (int rc = apply_plan(h, p)) return rc;
        *collapsed += n;
    }
    return GBG_OK;
}

// Glioma_HG_UQ::run (source/Glioma/Glioma_HG_UQ.cpp:511-582) on the block grid:
// the parameters rescaled and dt from the initial grid's spacing as the
// reference computes them, steps while t <= tend, a regrid (one refinement
// pass, then compression until it stops) whenever t reaches the next dump
// time, and the refinement after the loop.
int amr_run(Handle &h, const gbg_amr_run_opts &o, long *steps, int *regrids) {
    using clock = std::chrono::steady_clock;
    *steps = 0;
    *regrids = 0;
    gbg_amr_run_stats st{};
    st.min_blocks = st.max_blocks = h.amr.nb;
    double dt, Dw, Dg, rho = o.rho;
    reference_dt(BS * o.bpd, o.Dw_file, o.L, h.prec == GBG_PREC_F32REF, &dt, &Dw, &Dg, &rho);
    if (!h.amr.ghosts_valid)
        if (int rc = install_tables(h)) return rc;
    // a regrid, timed from the end of the steps before it
    auto regrid = [&](bool compress) -> int {
        GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
        const auto r0 = clock::now();
        int r = 0, c = 0;
        if (int rc = amr_auto_refine(h, o.refine_tol, o.max_level, &r)) return rc;
        if (compress)
            if (int rc = amr_auto_compress(h, o.compress_tol, &c)) return rc;
        st.regrid_seconds += std::chrono::duration<double>(clock::now() - r0).count();
        ++st.regrid_calls;
        ++*regrids;
        st.min_blocks = std::min(st.min_blocks, h.amr.nb);
        st.max_blocks = std::max(st.max_blocks, h.amr.nb);
        return GBG_OK;
    };
    const auto t0 = clock::now();
    double t = 0.0, when = o.dumpfreq;
    long k = 0;
    while (t <= o.tend && k < 100000000L) {
        if (int rc = amr_steps(h, Dw, Dg, rho, dt, 1)) return rc;
        st.cell_steps += (long long)h.amr.nb * BS * BS * BS;
        t += dt;
        ++k;
        if (t >= when) {
            if (o.adaptive)
                if (int rc = regrid(true)) return rc;
            when = when + o.dumpfreq;
        }
    }
    *steps = k;
    if (o.adaptive && o.final_refine)
        if (int rc = regrid(false)) return rc;
    GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    st.step_seconds = std::chrono::duration<double>(clock::now() - t0).count() - st.regrid_seconds;
    h.amr.last_run = st;
    return GBG_OK;
}

}  // namespace gbg

using gbg::set_error;

extern "C" {

int gbg_amr_ghost_tables(int nb, const gbg_block *blocks, long *start, int *src_block, int *src_cell, double *w,
                         long capacity, long *nentries) {
    if (nb < 1 || !blocks || !nentries || !start) {
        set_error("gbg_amr_ghost_tables: bad argument");
        return GBG_ERR_ARG;
    }
    gbg::Tree t;
    if (t.build(blocks, nb) != GBG_OK) {
        set_error("gbg_amr_ghost_tables: the blocks do not tile the unit cube as a block tree");
        return GBG_ERR_ARG;
    }
    gbg::Tables tb;
    if (int rc = gbg::compile_tables(t, tb)) return rc;
    *nentries = (long)tb.src_block.size();
    std::memcpy(start, tb.start.data(), tb.start.size() * sizeof(long));
    if (!src_block || !src_cell || !w) return GBG_OK;  // size query
    if (capacity < *nentries) {
        set_error("gbg_amr_ghost_tables: capacity below the table size (see *nentries)");
        return GBG_ERR_ARG;
    }
    std::memcpy(src_block, tb.src_block.data(), tb.src_block.size() * sizeof(int));
    std::memcpy(src_cell, tb.src_cell.data(), tb.src_cell.size() * sizeof(int));
    std::memcpy(w, tb.w.data(), tb.w.size() * sizeof(double));
    return GBG_OK;
}

static int copy_plan(const gbg::Plan &p, int capacity, gbg_block *blocks_new, int *kind, int *src, int *nb_new) {
    *nb_new = (int)p.blocks.size();
    if (capacity < *nb_new) {
        set_error("plan needs more blocks than the capacity (see *nb_new)");
        return GBG_ERR_ARG;
    }
    std::memcpy(blocks_new, p.blocks.data(), p.blocks.size() * sizeof(gbg_block));
    std::memcpy(kind, p.kind.data(), p.kind.size() * sizeof(int));
    std::memcpy(src, p.src.data(), p.src.size() * sizeof(int));
    return GBG_OK;
}

int gbg_amr_plan_refine(int nb, const gbg_block *blocks, const unsigned char *flagged, int max_level, int capacity,
                        gbg_block *blocks_new, int *kind, int *src, int *nb_new, int *nrefined) {
    if (nb < 1 || !blocks || !flagged || !blocks_new || !kind || !src || !nb_new || !nrefined) {
        set_error("gbg_amr_plan_refine: bad argument");
        return GBG_ERR_ARG;
    }
    gbg::Tree t;
    if (t.build(blocks, nb) != GBG_OK) {
        set_error("gbg_amr_plan_refine: the blocks do not tile the unit cube as a block tree");
        return GBG_ERR_ARG;
    }
    std::vector<char> f(flagged, flagged + nb);
    gbg::Plan p;
    *nrefined = gbg::plan_refine(t, f, max_level, p);
    return copy_plan(p, capacity, blocks_new, kind, src, nb_new);
}

int gbg_amr_plan_compress(int nb, const gbg_block *blocks, const unsigned char *flagged, int capacity,
                          gbg_block *blocks_new, int *kind, int *src, int *nb_new, int *ncollapsed) {
    if (nb < 1 || !blocks || !flagged || !blocks_new || !kind || !src || !nb_new || !ncollapsed) {
        set_error("gbg_amr_plan_compress: bad argument");
        return GBG_ERR_ARG;
    }
    gbg::Tree t;
    if (t.build(blocks, nb) != GBG_OK) {
        set_error("gbg_amr_plan_compress: the blocks do not tile the unit cube as a block tree");
        return GBG_ERR_ARG;
    }
    std::vector<char> f(flagged, flagged + nb);
    gbg::Plan p;
    *ncollapsed = gbg::plan_compress(t, f, p);
    return copy_plan(p, capacity, blocks_new, kind, src, nb_new);
}

}  // extern "C"
