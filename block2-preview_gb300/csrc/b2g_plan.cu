// Host-side plan builder: turns the recorded GEMM-pair sequence of one
// H_eff*psi (BatchGEMMSeq batch[0]/batch[1] after
// EffectiveHamiltonian::precompute, src/dmrg/effective_hamiltonian.hpp:226-246)
// into the device schedule executed by the phase-1/phase-2 kernels.
//
// What the reference does per Davidson iteration (Tasked replay,
// src/core/batch_gemm.hpp:1613-1689): every pair recomputes its own
// W = alpha0 * psi_sub * op(R) and accumulates alpha1 * op(L) * W into a
// per-thread copy of sigma, followed by a tree reduction of the copies.
// The plan removes both redundancies GPU-side:
//   * identical GEMM0 products (same psi sub-block, same operator block) are
//     computed once (alpha0 moves into the GEMM1 coefficient);
//   * sigma is cut into disjoint regions and tasks, each task owns its cells,
//     so no atomics, no sigma copies and no reduction are needed, and the
//     summation order is fixed (bit-reproducible run to run).
// For the tensor-core form it also lays out the operand images: GEMM0 tiles
// (products sharing a right operator, stacked psi rows, transposed), GEMM1
// tiles per sigma rectangle with one stage per 16-row K slab of each
// contribution, split-K chunks, and the cover lists of the reduction.
#include <algorithm>
#include <array>
#include <cstring>
#include <string>
#include <unordered_map>

#include "b2g_internal.h"

namespace b2g {

namespace {

struct WorkKey {
    uint64_t a0, b0;
    int32_t m0, n0, k0, lda0, ldb0, tb0;
    bool operator==(const WorkKey &o) const {
        return a0 == o.a0 && b0 == o.b0 && m0 == o.m0 && n0 == o.n0 && k0 == o.k0 &&
               lda0 == o.lda0 && ldb0 == o.ldb0 && tb0 == o.tb0;
    }
};
struct WorkKeyHash {
    size_t operator()(const WorkKey &k) const {
        uint64_t h = k.a0 * 0x9E3779B97F4A7C15ULL ^ (k.b0 + 0x632BE59BD9B4E019ULL);
        h ^= ((uint64_t)(uint32_t)k.m0 << 32 | (uint32_t)k.n0) * 0xBF58476D1CE4E5B9ULL;
        h ^= ((uint64_t)(uint32_t)k.k0 << 32 | (uint32_t)k.lda0) * 0x94D049BB133111EBULL;
        h ^= ((uint64_t)(uint32_t)k.ldb0 << 1 | (uint32_t)k.tb0) * 0xD6E8FEB86659FD93ULL;
        return (size_t)(h ^ (h >> 31));
    }
};

struct Rect4Hash {
    size_t operator()(const std::array<int32_t, 4> &k) const {
        uint64_t h = ((uint64_t)(uint32_t)k[0] << 32 | (uint32_t)k[1]) * 0x9E3779B97F4A7C15ULL;
        h ^= ((uint64_t)(uint32_t)k[2] << 32 | (uint32_t)k[3]) * 0xBF58476D1CE4E5B9ULL;
        return (size_t)(h ^ (h >> 31));
    }
};
struct Psi4Hash {
    size_t operator()(const std::array<int64_t, 4> &k) const {
        uint64_t h = (uint64_t)k[0] * 0x9E3779B97F4A7C15ULL;
        h ^= ((uint64_t)k[1] << 40 ^ (uint64_t)k[2] << 20 ^ (uint64_t)k[3]) * 0xBF58476D1CE4E5B9ULL;
        return (size_t)(h ^ (h >> 29));
    }
};

// extent in doubles of a row-major operand of logical shape rows x cols (after op)
inline uint64_t extent(bool trans, int64_t rows, int64_t cols, int64_t ld) {
    if (rows == 0 || cols == 0)
        return 0;
    return trans ? (uint64_t)((cols - 1) * ld + rows) : (uint64_t)((rows - 1) * ld + cols);
}

// off + ext <= size, in a form no caller-supplied offset can make wrap around
inline bool fits(uint64_t off, uint64_t ext, uint64_t size) { return ext <= size && off <= size - ext; }

} // namespace

static constexpr int kRowsPerTask = 4;    // warps per phase-2 CTA, one row each
static constexpr int kColsPerTask = 256;  // 8 x 32 lanes

int build_plan(const b2g_pair_seq *s, uint64_t ops_size, uint64_t psi_size, uint64_t sigma_size,
               HostPlan &plan, const PlanParams &params) {
    if (s == nullptr || s->n_pairs < 0)
        return fail(B2G_ERR_ARG, "b2g_heff_create: null or negative pair sequence");
    if ((params.g0_tile_cols != 128 && params.g0_tile_cols != 256) ||
        (params.g1_tile_cols != 128 && params.g1_tile_cols != 256) || params.g1_chunk < 1 ||
        params.g1_chunk > kG1ChunkLimit)
        return fail(B2G_ERR_ARG, "plan parameters outside the supported tile shapes");
    const int64_t np = s->n_pairs;
    plan = HostPlan();
    plan.params = params;
    const int32_t g1w = params.g1_tile_cols, g0w = params.g0_tile_cols;
    // ---- validation + GEMM0 de-duplication -------------------------------
    std::unordered_map<WorkKey, int32_t, WorkKeyHash> wmap;
    wmap.reserve((size_t)np * 2 + 1);
    std::vector<int32_t> pu(np, -1);
    std::vector<char> live(np, 0);
    for (int64_t i = 0; i < np; i++) {
        const int32_t m0 = s->m0[i], n0 = s->n0[i], k0 = s->k0[i];
        const int32_t m1 = s->m1[i], n1 = s->n1[i], k1 = s->k1[i];
        if (m0 < 0 || n0 < 0 || k0 < 0 || m1 < 0 || n1 < 0 || k1 < 0)
            return fail(B2G_ERR_ARG, "pair " + std::to_string(i) + ": negative dimension");
        if (k1 != m0 || n1 != n0)
            return fail(B2G_ERR_UNSUPPORTED,
                        "pair " + std::to_string(i) + ": GEMM1 does not consume the GEMM0 work matrix");
        if (m1 == 0 || n1 == 0 || k1 == 0 || k0 == 0)
            continue;  // contributes nothing
        if (s->lda0[i] < k0 || s->ldc1[i] < n1 || s->ldb0[i] < (s->tb0[i] ? k0 : n0) ||
            s->lda1[i] < (s->ta1[i] ? m1 : k1))
            return fail(B2G_ERR_ARG, "pair " + std::to_string(i) + ": leading dimension too small");
        if (!fits(s->a0[i], extent(false, m0, k0, s->lda0[i]), psi_size))
            return fail(B2G_ERR_ARG, "pair " + std::to_string(i) + ": psi operand out of range");
        if (!fits(s->b0[i], extent(s->tb0[i], k0, n0, s->ldb0[i]), ops_size))
            return fail(B2G_ERR_ARG, "pair " + std::to_string(i) + ": GEMM0 operator out of range");
        if (!fits(s->a1[i], extent(s->ta1[i], m1, k1, s->lda1[i]), ops_size))
            return fail(B2G_ERR_ARG, "pair " + std::to_string(i) + ": GEMM1 operator out of range");
        if (!fits(s->c1[i], extent(false, m1, n1, s->ldc1[i]), sigma_size))
            return fail(B2G_ERR_ARG, "pair " + std::to_string(i) + ": sigma operand out of range");
        live[i] = 1;
        plan.mnk += (double)m0 * n0 * k0 + (double)m1 * n1 * k1;
        WorkKey key{s->a0[i], s->b0[i], m0, n0, k0, s->lda0[i], s->ldb0[i], s->tb0[i] ? 1 : 0};
        auto it = wmap.find(key);
        if (it == wmap.end()) {
            const int32_t u = (int32_t)plan.works.size();
            wmap.emplace(key, u);
            WorkDesc wd;
            wd.a0 = key.a0, wd.b0 = key.b0, wd.woff = plan.work_size;
            wd.m0 = m0, wd.n0 = n0, wd.k0 = k0, wd.lda0 = key.lda0, wd.ldb0 = key.ldb0, wd.tb0 = key.tb0;
            plan.works.push_back(wd);
            plan.work_size += (uint64_t)m0 * n0;
            plan.mnk_exec += (double)m0 * n0 * k0;
            pu[i] = u;
        } else
            pu[i] = it->second;
        plan.mnk_exec += (double)m1 * n1 * k1;
    }
    // ---- sigma regions: merge overlapping write spans ---------------------
    std::vector<int64_t> order;
    order.reserve(np);
    for (int64_t i = 0; i < np; i++)
        if (live[i])
            order.push_back(i);
    std::sort(order.begin(), order.end(), [s](int64_t a, int64_t b) {
        return s->c1[a] != s->c1[b] ? s->c1[a] < s->c1[b] : a < b;
    });
    std::vector<std::vector<int64_t>> groups;
    uint64_t cur_end = 0;
    for (int64_t i : order) {
        const uint64_t st = s->c1[i], en = st + extent(false, s->m1[i], s->n1[i], s->ldc1[i]);
        if (groups.empty() || st >= cur_end) {
            groups.emplace_back();
            cur_end = en;
        } else
            cur_end = std::max(cur_end, en);
        groups.back().push_back(i);
    }
    // ---- per region: a non-wrapping column frame, placements, tasks --------
    std::vector<int32_t> cover;
    for (auto &gp : groups) {
        const int32_t ld = s->ldc1[gp[0]];
        for (int64_t i : gp)
            if (s->ldc1[i] != ld)
                return fail(B2G_ERR_UNSUPPORTED, "sigma region written with two leading dimensions");
        // interior coverage on the circle of length ld: a frame cut at x is valid
        // when no write window [r, r+n) contains x strictly inside.
        cover.assign((size_t)ld + 1, 0);
        for (int64_t i : gp) {
            const int64_t r = (int64_t)(s->c1[i] % (uint64_t)ld), n = s->n1[i];
            for (int64_t j = 1; j < n; j++)
                cover[(size_t)((r + j) % ld)] = 1;
        }
        int32_t cut = -1;
        for (int32_t x = 0; x < ld; x++)
            if (!cover[x]) {
                cut = x;
                break;
            }
        if (cut < 0)
            return fail(B2G_ERR_UNSUPPORTED, "no consistent column frame for a sigma region");
        Region rg;
        rg.ld = ld, rg.pad = 0;
        rg.lo = UINT64_MAX, rg.hi = 0;
        for (int64_t i : gp) {
            rg.lo = std::min(rg.lo, s->c1[i]);
            rg.hi = std::max(rg.hi, s->c1[i] + extent(false, s->m1[i], s->n1[i], s->ldc1[i]));
        }
        uint64_t base = UINT64_MAX;
        std::vector<int64_t> colp(gp.size());
        for (size_t q = 0; q < gp.size(); q++) {
            const int64_t i = gp[q];
            const int64_t r = (int64_t)(s->c1[i] % (uint64_t)ld);
            colp[q] = ((r - cut) % ld + ld) % ld;
            base = std::min(base, s->c1[i] - (uint64_t)colp[q]);
        }
        rg.base = base;
        int32_t rows = 0, cols = 0;
        const int32_t g = (int32_t)plan.regions.size();
        const size_t c_begin = plan.contribs.size();
        for (size_t q = 0; q < gp.size(); q++) {
            const int64_t i = gp[q];
            Contrib c;
            c.a1 = s->a1[i];
            c.alpha = s->alpha0[i] * s->alpha1[i];
            c.u = pu[i];
            c.col0 = (int32_t)colp[q];
            c.row0 = (int32_t)((s->c1[i] - (uint64_t)colp[q] - base) / (uint64_t)ld);
            c.m1 = s->m1[i], c.n1 = s->n1[i], c.k1 = s->k1[i];
            c.lda1 = s->lda1[i], c.ta1 = s->ta1[i] ? 1 : 0;
            if (c.col0 + c.n1 > ld)
                return fail(B2G_ERR_UNSUPPORTED, "sigma write window wraps its region frame");
            rows = std::max(rows, c.row0 + c.m1);
            cols = std::max(cols, c.col0 + c.n1);
            plan.contribs.push_back(c);
        }
        rg.rows = rows, rg.cols = cols;
        plan.regions.push_back(rg);
        plan.region_cb.push_back((int64_t)c_begin);
        const int32_t nrb = (rows + kRowsPerTask - 1) / kRowsPerTask;
        const int32_t ncs = (cols + kColsPerTask - 1) / kColsPerTask;
        std::vector<std::vector<int32_t>> tl((size_t)nrb * ncs);
        for (size_t q = c_begin; q < plan.contribs.size(); q++) {
            const Contrib &c = plan.contribs[q];
            const int32_t rb0 = c.row0 / kRowsPerTask, rb1 = (c.row0 + c.m1 - 1) / kRowsPerTask;
            const int32_t cs0 = c.col0 / kColsPerTask, cs1 = (c.col0 + c.n1 - 1) / kColsPerTask;
            for (int32_t rb = rb0; rb <= rb1; rb++)
                for (int32_t cs = cs0; cs <= cs1; cs++)
                    tl[(size_t)rb * ncs + cs].push_back((int32_t)q);
        }
        for (int32_t rb = 0; rb < nrb; rb++)
            for (int32_t cs = 0; cs < ncs; cs++) {
                auto &l = tl[(size_t)rb * ncs + cs];
                if (l.empty())
                    continue;
                // split the list into chunks of at most kSimtChunkK k-steps
                const int64_t lb = (int64_t)plan.lists.size();
                plan.lists.insert(plan.lists.end(), l.begin(), l.end());
                std::vector<int64_t> cuts{lb};
                int64_t acc = 0;
                for (size_t q = 0; q < l.size(); q++) {
                    const int32_t k = plan.contribs[l[q]].k1;
                    if (acc > 0 && acc + k > kSimtChunkK) {
                        cuts.push_back(lb + (int64_t)q);
                        acc = 0;
                    }
                    acc += k;
                }
                cuts.push_back(lb + (int64_t)l.size());
                const int32_t nch = (int32_t)cuts.size() - 1;
                int64_t part = -1;
                if (nch > 1) {
                    part = (int64_t)plan.t2_part_tiles;
                    plan.t2_part_tiles += (uint64_t)nch;
                    plan.t2multi.push_back(Tile2{g, rb, cs * kColsPerTask, nch, part});
                }
                for (int32_t ch = 0; ch < nch; ch++) {
                    Task2 t;
                    t.g = g, t.rb = rb, t.col0 = cs * kColsPerTask, t.chunk = ch;
                    t.lb = cuts[ch], t.le = cuts[ch + 1], t.part = part;
                    plan.t2.push_back(t);
                }
            }
        // image-fed tensor-core GEMM1: one tile per 128-row x 256-column piece of
        // each distinct sigma rectangle, one stage per 16-row K slab of each
        // contribution (stage offsets into the A / W images filled in below)
        {
            std::vector<std::array<int32_t, 4>> rkeys;   // rectangles, first-appearance order
            std::unordered_map<std::array<int32_t, 4>, int32_t, Rect4Hash> rmap;
            std::vector<std::vector<int32_t>> rlist;
            for (size_t q = c_begin; q < plan.contribs.size(); q++) {
                const Contrib &c = plan.contribs[q];
                const std::array<int32_t, 4> rk{c.row0, c.m1, c.col0, c.n1};
                auto it = rmap.find(rk);
                if (it == rmap.end()) {
                    it = rmap.emplace(rk, (int32_t)rkeys.size()).first;
                    rkeys.push_back(rk);
                    rlist.emplace_back();
                }
                rlist[it->second].push_back((int32_t)q);
            }
            const int32_t t_first = (int32_t)plan.g1tile.size();
            for (size_t z = 0; z < rkeys.size(); z++) {
                const int32_t row0 = rkeys[z][0], m1 = rkeys[z][1], col0 = rkeys[z][2], n1 = rkeys[z][3];
                const int32_t npad = (n1 + 15) / 16 * 16;
                for (int32_t rp = 0; rp * 128 < m1; rp++)
                    for (int32_t cp = 0; cp * g1w < npad; cp++) {
                        G1Tile t;
                        t.g = g, t.row0 = row0 + 128 * rp, t.col0 = col0 + g1w * cp;
                        t.rows = std::min(128, m1 - 128 * rp);
                        t.n = std::min(g1w, npad - g1w * cp);
                        t.ncols = std::min(t.n, n1 - g1w * cp);
                        t.pad = 0;
                        t.n_chunks = 0;
                        t.part = (int64_t)plan.g1stage.size();  // first stage until chunking
                        for (int32_t q : rlist[z]) {
                            const Contrib &c = plan.contribs[q];
                            const int32_t nsl = (c.k1 + kG1SlabK - 1) / kG1SlabK;
                            for (int32_t sl = 0; sl < nsl; sl++) {
                                G1Stage st;
                                // a: A image id / piece / slab, b: work id / slab / column piece
                                st.a = (uint64_t)q;
                                st.b = ((uint64_t)(uint32_t)sl << 32) | (uint32_t)(rp << 16 | cp);
                                st.a_bytes = 0, st.b_lo = 0;
                                plan.g1stage.push_back(st);
                            }
                        }
                        plan.g1tile.push_back(t);
                    }
            }
            const int32_t t_last = (int32_t)plan.g1tile.size();
            // reduction items: 4 region rows each (enough CTAs to keep the chunk
            // loads in flight), with the tiles meeting those rows in tile order
            // (each tile is added to the items its rows meet)
            const int32_t nitems = (rows + 3) / 4;
            std::vector<std::vector<int32_t>> cover((size_t)nitems);
            for (int32_t t = t_first; t < t_last; t++) {
                const G1Tile &tt = plan.g1tile[t];
                const int32_t i0 = std::max(0, tt.row0) / 4;
                const int32_t i1 = std::min(nitems - 1, (tt.row0 + tt.rows - 1) / 4);
                for (int32_t i = i0; i <= i1; i++)
                    cover[(size_t)i].push_back(t);
            }
            for (int32_t i = 0; i < nitems; i++) {
                G1Red it;
                it.g = g, it.r0 = 4 * i, it.r1 = std::min(rows, 4 * i + 4);
                it.t0 = (int32_t)plan.g1cover.size();
                plan.g1cover.insert(plan.g1cover.end(), cover[(size_t)i].begin(), cover[(size_t)i].end());
                it.t1 = (int32_t)plan.g1cover.size(), it.pad = 0;
                if (it.t1 > it.t0)
                    plan.g1red.push_back(it);
            }
        }
    }
    plan.region_cb.push_back((int64_t)plan.contribs.size());
    // ---- diagonal tasks: a contribution reaches diag(H_eff) only where its
    // psi sub-block and its sigma sub-block share offsets, i.e. inside its
    // sigma rectangle and on the rows of the region frame that the flat
    // overlap [max(x0, y0), min(x1, y1)) spans (a conservative cell set; the
    // diag kernel applies the exact index test).  Each region is cut into
    // tiles of kDiagTileRows x kDiagTileCols cells; a tile lists the
    // contributions whose cell set meets it, in contribution order.
    {
        std::vector<std::vector<int32_t>> tile;
        for (size_t g = 0; g < plan.regions.size(); g++) {
            const Region &rg = plan.regions[g];
            if (rg.rows <= 0 || rg.cols <= 0)
                continue;
            const int32_t nrb = (rg.rows + kDiagTileRows - 1) / kDiagTileRows;
            const int32_t ncb = (rg.cols + kDiagTileCols - 1) / kDiagTileCols;
            tile.assign((size_t)nrb * ncb, std::vector<int32_t>());
            for (int64_t q = plan.region_cb[g]; q < plan.region_cb[g + 1]; q++) {
                const Contrib &ct = plan.contribs[q];
                const WorkDesc &w = plan.works[ct.u];
                const uint64_t x0 = rg.base + (uint64_t)ct.row0 * rg.ld + (uint64_t)ct.col0;
                const uint64_t x1 = x0 + (uint64_t)(ct.m1 - 1) * rg.ld + (uint64_t)ct.n1;
                const uint64_t y0 = w.a0, y1 = w.a0 + extent(false, w.m0, w.k0, w.lda0);
                if (!(x0 < y1 && y0 < x1))
                    continue;
                DiagItem it;
                it.a1 = ct.a1, it.b0 = w.b0, it.a0 = w.a0, it.alpha = ct.alpha;
                it.row0 = ct.row0, it.col0 = ct.col0, it.m1 = ct.m1, it.n1 = ct.n1;
                it.m0 = w.m0, it.k0 = w.k0, it.lda0 = w.lda0, it.lda1 = ct.lda1, it.ldb0 = w.ldb0;
                it.ta1 = (int16_t)ct.ta1, it.tb0 = (int16_t)w.tb0, it.pad = 0;
                it.same_ld = w.lda0 == rg.ld ? 1 : 0, it.ra = 0, it.ca = 0;
                if (it.same_ld) {
                    // floor division of the (possibly negative) frame offset of a0
                    const int64_t d = (int64_t)w.a0 - (int64_t)rg.base;
                    const int64_t ra = d >= 0 ? d / rg.ld : -((-d + rg.ld - 1) / rg.ld);
                    it.ra = (int32_t)ra, it.ca = (int32_t)(d - ra * rg.ld);
                }
                const int32_t item = (int32_t)plan.diag_item.size();
                plan.diag_item.push_back(it);
                const uint64_t lo = std::max(x0, y0), hi = std::min(x1, y1);
                int64_t r_lo = (int64_t)((lo - rg.base) / (uint64_t)rg.ld);
                int64_t r_hi = (int64_t)((hi - 1 - rg.base) / (uint64_t)rg.ld) + 1;
                r_lo = std::max<int64_t>(r_lo, ct.row0);
                r_hi = std::min<int64_t>(r_hi, (int64_t)ct.row0 + ct.m1);
                const int64_t cb0 = ct.col0 / kDiagTileCols, cb1 = (ct.col0 + ct.n1 - 1) / kDiagTileCols;
                for (int64_t rb = r_lo / kDiagTileRows; rb < nrb && rb * kDiagTileRows < r_hi; rb++)
                    for (int64_t cb = cb0; cb <= cb1 && cb < ncb; cb++)
                        tile[(size_t)(rb * ncb + cb)].push_back(item);
            }
            for (int32_t rb = 0; rb < nrb; rb++)
                for (int32_t cb = 0; cb < ncb; cb++) {
                    const auto &l = tile[(size_t)rb * ncb + cb];
                    if (l.empty())
                        continue;
                    DiagTask t;
                    t.g = (int32_t)g, t.pad = 0;
                    t.r0 = rb * kDiagTileRows, t.r1 = std::min(rg.rows, (rb + 1) * kDiagTileRows);
                    t.c0 = cb * kDiagTileCols, t.c1 = std::min(rg.cols, (cb + 1) * kDiagTileCols);
                    t.lb = (int64_t)plan.diag_tlist.size();
                    plan.diag_tlist.insert(plan.diag_tlist.end(), l.begin(), l.end());
                    t.le = (int64_t)plan.diag_tlist.size();
                    plan.diag_task.push_back(t);
                }
        }
    }
    // ---- image-fed GEMM1: A images (one per distinct operator block and
    // coefficient), W image offsets, stage byte offsets, split-K chunks
    {
        struct AKey {
            uint64_t a1;
            int32_t m1, k1, lda1, ta1;
            float alpha;
            bool operator==(const AKey &o) const {
                return a1 == o.a1 && m1 == o.m1 && k1 == o.k1 && lda1 == o.lda1 && ta1 == o.ta1 &&
                       memcmp(&alpha, &o.alpha, sizeof(float)) == 0;
            }
        };
        struct AKeyHash {
            size_t operator()(const AKey &k) const {
                uint32_t ab;
                memcpy(&ab, &k.alpha, sizeof ab);
                uint64_t h = k.a1 * 0x9E3779B97F4A7C15ULL;
                h ^= ((uint64_t)(uint32_t)k.m1 << 32 | (uint32_t)k.k1) * 0xBF58476D1CE4E5B9ULL;
                h ^= ((uint64_t)(uint32_t)k.lda1 << 33 | (uint64_t)k.ta1 << 32 | ab) * 0x94D049BB133111EBULL;
                return (size_t)(h ^ (h >> 29));
            }
        };
        std::unordered_map<AKey, int32_t, AKeyHash> amap;
        std::vector<int32_t> cimg(plan.contribs.size(), -1);
        for (size_t q = 0; q < plan.contribs.size(); q++) {
            const Contrib &c = plan.contribs[q];
            AKey k{c.a1, c.m1, c.k1, c.lda1, c.ta1, (float)c.alpha};
            auto it = amap.find(k);
            if (it == amap.end()) {
                G1AImg im;
                im.src = c.a1, im.dst = plan.g1_abytes, im.alpha = (float)c.alpha;
                im.m1 = c.m1, im.k1 = c.k1, im.lda1 = c.lda1, im.ta1 = c.ta1, im.pad = 0;
                const uint64_t nsl = (uint64_t)((c.k1 + kG1SlabK - 1) / kG1SlabK);
                for (int32_t rp = 0; rp * 128 < c.m1; rp++) {
                    const int32_t rows8 = (std::min(128, c.m1 - 128 * rp) + 7) / 8 * 8;
                    plan.g1_abytes += (uint64_t)rows8 * 128 * nsl;
                }
                it = amap.emplace(k, (int32_t)plan.g1aimg.size()).first;
                plan.g1aimg.push_back(im);
            }
            cimg[q] = it->second;
        }
        std::vector<uint64_t> wdst(plan.works.size());
        for (size_t u = 0; u < plan.works.size(); u++) {
            const WorkDesc &w = plan.works[u];
            const int32_t npad = (w.n0 + 15) / 16 * 16;
            G1WImg wi;
            wi.dst = plan.g1_wbytes, wi.u = (int32_t)u, wi.npad = npad;
            wdst[u] = wi.dst;
            plan.g1wimg.push_back(wi);
            plan.g1_wbytes += (uint64_t)((w.m0 + kG1SlabK - 1) / kG1SlabK) * npad * 128;
        }
        for (G1Stage &st : plan.g1stage) {
            const Contrib &c = plan.contribs[(size_t)st.a];
            const G1AImg &im = plan.g1aimg[cimg[(size_t)st.a]];
            const int32_t sl = (int32_t)(st.b >> 32), rp = (int32_t)((st.b >> 16) & 0xFFFF),
                          cp = (int32_t)(st.b & 0xFFFF);
            const uint64_t nsl = (uint64_t)((c.k1 + kG1SlabK - 1) / kG1SlabK);
            const int32_t rows8 = (std::min(128, c.m1 - 128 * rp) + 7) / 8 * 8;
            const WorkDesc &w = plan.works[c.u];
            const int32_t npad = (w.n0 + 15) / 16 * 16;
            st.a = im.dst + (uint64_t)rp * 16384 * nsl + (uint64_t)sl * rows8 * 128;
            st.a_bytes = (uint32_t)rows8 * 64;
            st.b = wdst[c.u] + (uint64_t)sl * npad * 128 + (uint64_t)cp * g1w * 64;
            st.b_lo = (uint32_t)npad * 64;
        }
        for (int32_t t = 0; t < (int32_t)plan.g1tile.size(); t++) {
            G1Tile &tl = plan.g1tile[t];
            const int64_t sb = tl.part;
            const int64_t se = t + 1 < (int32_t)plan.g1tile.size() ? plan.g1tile[t + 1].part
                                                                   : (int64_t)plan.g1stage.size();
            int32_t ch = 0;
            for (int64_t st = sb; st < se; st += params.g1_chunk, ch++) {
                G1Task k;
                k.tile = t, k.chunk = ch, k.st0 = st;
                k.n_stages = (int32_t)std::min<int64_t>(params.g1_chunk, se - st), k.pad = 0;
                plan.g1task.push_back(k);
            }
            tl.n_chunks = ch;
        }
        for (G1Tile &tl : plan.g1tile) {
            tl.part = (int64_t)plan.g1_part;
            plan.g1_part += (uint64_t)tl.n_chunks * tl.rows * tl.n;
        }
        std::stable_sort(plan.g1task.begin(), plan.g1task.end(),
                         [](const G1Task &a, const G1Task &b) { return a.n_stages > b.n_stages; });
    }
    // heavy tasks first: shortens the tail of the phase-2 grid
    std::stable_sort(plan.t2.begin(), plan.t2.end(),
                     [](const Task2 &a, const Task2 &b) { return a.le - a.lb > b.le - b.lb; });
    size_t nt1 = 0;
    for (const WorkDesc &w : plan.works)
        nt1 += (size_t)w.m0;
    plan.t1.reserve(nt1);
    for (int32_t u = 0; u < (int32_t)plan.works.size(); u++)
        for (int32_t r = 0; r < plan.works[u].m0; r++)
            plan.t1.push_back(Task1{u, r});
    // ---- tensor-core GEMM0 (transposed): op(R)^T pieces x stacked psi rows of
    // the products sharing R; op(R)^T images join the A image buffer
    {
        std::vector<int32_t> ord(plan.works.size());
        for (size_t i = 0; i < ord.size(); i++)
            ord[i] = (int32_t)i;
        auto key_less = [&](int32_t x, int32_t y) {
            const WorkDesc &a = plan.works[x], &b = plan.works[y];
            if (a.b0 != b.b0) return a.b0 < b.b0;
            if (a.tb0 != b.tb0) return a.tb0 < b.tb0;
            if (a.k0 != b.k0) return a.k0 < b.k0;
            if (a.n0 != b.n0) return a.n0 < b.n0;
            if (a.ldb0 != b.ldb0) return a.ldb0 < b.ldb0;
            return x < y;
        };
        std::sort(ord.begin(), ord.end(), key_less);
        auto same_r = [&](int32_t x, int32_t y) {
            const WorkDesc &a = plan.works[x], &b = plan.works[y];
            return a.b0 == b.b0 && a.tb0 == b.tb0 && a.k0 == b.k0 && a.n0 == b.n0 && a.ldb0 == b.ldb0;
        };
        std::unordered_map<std::array<int64_t, 4>, int32_t, Psi4Hash> pmap;  // distinct psi sub-blocks
        pmap.reserve(plan.works.size() + 1);
        size_t nrows = 0;   // stacked psi rows of all tiles (each product padded to 4)
        for (const WorkDesc &w : plan.works)
            nrows += (size_t)((w.m0 + 3) / 4 * 4);
        plan.g0col.reserve(plan.g0col.size() + nrows);
        for (size_t gs = 0; gs < ord.size();) {
            size_t ge = gs + 1;
            while (ge < ord.size() && same_r(ord[gs], ord[ge]))
                ge++;
            const WorkDesc &w0 = plan.works[ord[gs]];
            // the op(R)^T image: rows = the n0 columns of R, K = k0
            G1AImg im;
            im.src = w0.b0, im.dst = plan.g1_abytes, im.alpha = 1.0f;
            im.m1 = w0.n0, im.k1 = w0.k0, im.lda1 = w0.ldb0, im.ta1 = w0.tb0 ? 0 : 1, im.pad = 0;
            const int32_t nsl = (w0.k0 + kG1SlabK - 1) / kG1SlabK;
            for (int32_t rp = 0; rp * 128 < w0.n0; rp++) {
                const int32_t rows8 = (std::min(128, w0.n0 - 128 * rp) + 7) / 8 * 8;
                plan.g1_abytes += (uint64_t)rows8 * 128 * nsl;
            }
            plan.g1aimg.push_back(im);
            // stacked psi rows, each product padded to a multiple of 4; the rows
            // point into the packed copy of their psi sub-block
            const size_t col_begin = plan.g0col.size();
            for (size_t q = gs; q < ge; q++) {
                const int32_t u = ord[q];
                const WorkDesc &w = plan.works[u];
                const std::array<int64_t, 4> pk{(int64_t)w.a0, w.m0, w.k0, w.lda0};
                auto pit = pmap.find(pk);
                if (pit == pmap.end()) {
                    G0Psi ps;
                    ps.src = w.a0, ps.dst = plan.g0_psi_floats;
                    ps.m0 = w.m0, ps.k0 = w.k0, ps.lda0 = w.lda0, ps.k0p = (w.k0 + 3) / 4 * 4;
                    plan.g0_psi_floats += (uint64_t)ps.m0 * ps.k0p;
                    pit = pmap.emplace(pk, (int32_t)plan.g0psi.size()).first;
                    plan.g0psi.push_back(ps);
                }
                const G0Psi &ps = plan.g0psi[pit->second];
                const int32_t m0p = (w.m0 + 3) / 4 * 4;
                for (int32_t i = 0; i < m0p; i++) {
                    G0Col c;
                    c.psi = i < w.m0 ? ps.dst + (uint64_t)i * ps.k0p : 0;
                    c.w = plan.g1wimg[u].dst, c.k = i, c.live = i < w.m0 ? 1 : 0;
                    plan.g0col.push_back(c);
                }
            }
            const int32_t npad = (w0.n0 + 15) / 16 * 16;
            const size_t ncols = plan.g0col.size() - col_begin;
            for (size_t c0 = 0; c0 < ncols; c0 += (size_t)g0w) {
                const int32_t nc = (int32_t)std::min<size_t>((size_t)g0w, ncols - c0);
                const int64_t cb = (int64_t)(col_begin + c0);
                for (int32_t rp = 0; rp * 128 < w0.n0; rp++) {
                    G0Tile t;
                    t.rows = std::min(128, w0.n0 - 128 * rp);
                    const uint32_t rows8 = (uint32_t)(t.rows + 7) / 8 * 8;
                    t.a = im.dst + (uint64_t)rp * 16384 * nsl, t.a_bytes = rows8 * 64, t.nsl = nsl;
                    t.n = (nc + 15) / 16 * 16, t.ncol = nc;
                    t.k0 = w0.k0, t.npad = npad, t.m_off = 128 * rp, t.cb = cb;
                    plan.g0tile.push_back(t);
                }
            }
            gs = ge;
        }
        // wide tiles (N > 128) first, each class longest first
        std::stable_sort(plan.g0tile.begin(), plan.g0tile.end(), [](const G0Tile &a, const G0Tile &b) {
            const bool wa = a.n > 128, wb = b.n > 128;
            if (wa != wb)
                return wa;
            return (int64_t)a.nsl * a.n > (int64_t)b.nsl * b.n;
        });
        plan.g0_wide = 0;
        while (plan.g0_wide < (int64_t)plan.g0tile.size() && plan.g0tile[plan.g0_wide].n > 128)
            plan.g0_wide++;
    }
    return B2G_OK;
}

} // namespace b2g
