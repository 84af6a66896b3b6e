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
#include <algorithm>
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

// extent in doubles of a row-major operand of logical shape rows x cols (after op)
inline uint64_t extent(bool trans, int64_t rows, int64_t cols, int64_t ld) {
    if (rows == 0 || cols == 0)
        return 0;
    return trans ? (uint64_t)((cols - 1) * ld + rows) : (uint64_t)((rows - 1) * ld + cols);
}

} // namespace

static constexpr int kRowsPerTask = 4;    // warps per phase-2 CTA, one row each
static constexpr int kColsPerTask = 256;  // 8 x 32 lanes

int build_plan(const b2g_pair_seq *s, uint64_t ops_size, uint64_t psi_size, uint64_t sigma_size,
               HostPlan &plan) {
    if (s == nullptr || s->n_pairs < 0)
        return fail(B2G_ERR_ARG, "b2g_heff_create: null or negative pair sequence");
    const int64_t np = s->n_pairs;
    plan = HostPlan();
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
        if (s->a0[i] + extent(false, m0, k0, s->lda0[i]) > psi_size)
            return fail(B2G_ERR_ARG, "pair " + std::to_string(i) + ": psi operand out of range");
        if (s->b0[i] + extent(s->tb0[i], k0, n0, s->ldb0[i]) > ops_size)
            return fail(B2G_ERR_ARG, "pair " + std::to_string(i) + ": GEMM0 operator out of range");
        if (s->a1[i] + extent(s->ta1[i], m1, k1, s->lda1[i]) > ops_size)
            return fail(B2G_ERR_ARG, "pair " + std::to_string(i) + ": GEMM1 operator out of range");
        if (s->c1[i] + extent(false, m1, n1, s->ldc1[i]) > sigma_size)
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
        // tensor-core tiles: 128 rows x up to 256 columns, contributions packed
        // along K into stages of kTcStageK columns
        for (int32_t r0 = 0; r0 < rows; r0 += 128)
            for (int32_t c0 = 0; c0 < cols; c0 += 256) {
                const int32_t nt = std::min(256, ((cols - c0) + 15) / 16 * 16);
                const int64_t sb = (int64_t)plan.tcs.size();
                int32_t stage = 0, koff = 0;
                for (size_t q = c_begin; q < plan.contribs.size(); q++) {
                    const Contrib &c = plan.contribs[q];
                    if (c.row0 >= r0 + 128 || c.row0 + c.m1 <= r0 || c.col0 >= c0 + nt ||
                        c.col0 + c.n1 <= c0)
                        continue;
                    for (int32_t kb = 0; kb < c.k1;) {
                        const int32_t take = std::min(c.k1 - kb, kTcStageK - koff);
                        TcSeg sg;
                        sg.a = c.a1, sg.w = plan.works[c.u].woff, sg.alpha = (float)c.alpha;
                        sg.lda1 = c.lda1, sg.row0 = c.row0, sg.m1 = c.m1, sg.col0 = c.col0, sg.n1 = c.n1;
                        sg.kb = (int16_t)kb, sg.kl = (int16_t)take;
                        sg.koff = (int8_t)koff, sg.ta1 = (int8_t)c.ta1, sg.pad0 = 0, sg.pad1 = 0;
                        sg.stage = stage;
                        plan.tcs.push_back(sg);
                        kb += take, koff += take;
                        if (koff == kTcStageK)
                            stage++, koff = 0;
                    }
                }
                const int64_t se = (int64_t)plan.tcs.size();
                const int32_t n_stages = stage + (koff > 0 ? 1 : 0);
                if (se == sb)
                    continue;
                TcTile tl;
                tl.g = g, tl.row0 = r0, tl.col0 = c0, tl.n = nt;
                tl.rows = std::min(128, rows - r0);
                tl.n_chunks = n_stages;  // stage count until the chunking pass below
                tl.part = sb;            // segment start until the chunking pass below
                plan.tctile.push_back(tl);
            }
    }
    // ---- split-K chunking of the tensor-core tiles
    {
        int64_t total_stages = 0;
        for (auto &tl : plan.tctile)
            total_stages += tl.n_chunks;
        const int32_t chunk_stages = (int32_t)std::min<int64_t>(
            kTcMaxChunkStages,
            std::max<int64_t>(8, (total_stages + kTcTargetChunks - 1) / kTcTargetChunks));
        for (int32_t tile = 0; tile < (int32_t)plan.tctile.size(); tile++) {
            TcTile &tl = plan.tctile[tile];
            const int32_t n_stages = tl.n_chunks;
            const int64_t sb = tl.part;
            const int64_t se = tile + 1 < (int32_t)plan.tctile.size() ? plan.tctile[tile + 1].part
                                                                      : (int64_t)plan.tcs.size();
            std::vector<TcTask> chunks;
            int64_t s = sb;
            int32_t st = 0;
            while (st < n_stages) {
                TcTask t;
                t.tile = tile, t.chunk = (int32_t)chunks.size(), t.st0 = st, t.sb = s;
                // up to chunk_stages stages and kTcMaxSegs segments, whole stages only
                int32_t ns = 0;
                while (st + ns < n_stages && ns < chunk_stages) {
                    int64_t e = s;
                    while (e < se && plan.tcs[e].stage == st + ns)
                        e++;
                    if (ns > 0 && e - t.sb > kTcMaxSegs)
                        break;
                    s = e, ns++;
                }
                t.n_stages = ns, t.se = s;
                st += ns;
                chunks.push_back(t);
            }
            tl.n_chunks = (int32_t)chunks.size();
            tl.part = -1;
            if (tl.n_chunks > 1) {
                tl.part = (int64_t)plan.tc_part_size;
                plan.tc_part_size += (uint64_t)tl.n_chunks * tl.rows * tl.n;
                plan.tc_multi.push_back(tile);
            }
            plan.tct.insert(plan.tct.end(), chunks.begin(), chunks.end());
        }
    }
    std::stable_sort(plan.tct.begin(), plan.tct.end(),
                     [](const TcTask &a, const TcTask &b) { return a.n_stages > b.n_stages; });
    // heavy tasks first: shortens the tail of the phase-2 grid
    std::stable_sort(plan.t2.begin(), plan.t2.end(),
                     [](const Task2 &a, const Task2 &b) { return a.le - a.lb > b.le - b.lb; });
    for (int32_t u = 0; u < (int32_t)plan.works.size(); u++)
        for (int32_t r = 0; r < plan.works[u].m0; r++)
            plan.t1.push_back(Task1{u, r});
    // ---- tensor-core phase 1: stack rows of products sharing a right operator block
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
        for (size_t gs = 0; gs < ord.size();) {
            size_t ge = gs + 1;
            while (ge < ord.size() && same_r(ord[gs], ord[ge]))
                ge++;
            const WorkDesc &w0 = plan.works[ord[gs]];
            // rows of the group in order, cut into tiles of 128
            std::vector<Tc1Row> rows;
            for (size_t q = gs; q < ge; q++) {
                const WorkDesc &w = plan.works[ord[q]];
                for (int32_t r = 0; r < w.m0; r++)
                    rows.push_back(Tc1Row{w.a0 + (uint64_t)r * w.lda0, w.woff + (uint64_t)r * w.n0});
            }
            for (size_t r0 = 0; r0 < rows.size(); r0 += 128) {
                const int64_t rb = (int64_t)plan.tc1r.size();
                const int32_t nr = (int32_t)std::min<size_t>(128, rows.size() - r0);
                plan.tc1r.insert(plan.tc1r.end(), rows.begin() + r0, rows.begin() + r0 + nr);
                for (int32_t c0 = 0; c0 < w0.n0; c0 += 256) {
                    Tc1Tile t;
                    t.b0 = w0.b0, t.tb0 = w0.tb0, t.k0 = w0.k0, t.n0 = w0.n0, t.ldb0 = w0.ldb0;
                    t.col0 = c0, t.n = std::min(256, (w0.n0 - c0 + 15) / 16 * 16);
                    t.rows = nr, t.pad = 0, t.rb = rb;
                    plan.tc1t.push_back(t);
                }
            }
            gs = ge;
        }
        std::stable_sort(plan.tc1t.begin(), plan.tc1t.end(),
                         [](const Tc1Tile &a, const Tc1Tile &b) { return a.k0 * a.n > b.k0 * b.n; });
    }
    return B2G_OK;
}

} // namespace b2g
