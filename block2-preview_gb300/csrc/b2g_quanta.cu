// Quantum-number bookkeeping of the two-site wavefunction (host only,
// integer arithmetic, bit-exact with the reference):
//   * packed 64-bit labels: SZLongLong (src/core/symmetry.hpp:656-735) and
//     SU2LongLong (src/core/symmetry.hpp:1185-1300): +, unary -, the spin
//     range of a coupled label ([k], count), get_ket, get_bra, combine;
//   * StateInfo::tensor_product with a reference StateInfo or a target
//     filter, sort_states / collect, and get_connection_info
//     (src/core/state_info.hpp:160-310);
//   * SparseMatrixInfo::initialize for an operator or a wavefunction and
//     initialize_block_shifts / get_total_memory
//     (src/core/sparse_matrix.hpp:617-630, 727-757, 804-820);
//   * the wavefunction connection info of an effective Hamiltonian
//     (ConnectionInfo::initialize_wfn, src/core/sparse_matrix.hpp:163-292)
//     with SU(2) recoupling factors (9j symbols from Racah's 6j formula,
//     transposition factors) computed in long double.
// The label layouts and the carry/borrow behaviour of the packed arithmetic
// are part of the reference's data format (labels are compared as raw 64-bit
// words and stored in block lists), so the word-level operations are the
// same; everything around them is written for this library.
#include <algorithm>
#include <map>
#include <string>
#include <vector>

#include "b2g_internal.h"

namespace b2g {
namespace {

constexpr uint64_t kInvalid = ~0ULL;
constexpr uint64_t kTop16 = 0xFFFF000000000000ULL;   // particle number
constexpr uint64_t kPg = 0xFFFFULL;                  // point group irrep
constexpr uint64_t kSumFields = 0xFFFF0000FFFF0000ULL;

// ---- SZLongLong: N (16 bits, signed) | 0 (16) | 2Sz (16, signed) | pg (16)
struct Sz {
    static uint64_t neg(uint64_t a) {
        return (a & kPg) | ((~a + (1ULL << 16)) & 0xFFFF0000ULL) | ((~a + (1ULL << 48)) & kTop16);
    }
    static uint64_t add(uint64_t a, uint64_t b) {
        return (((a & kSumFields) + (b & kSumFields)) & kSumFields) | ((a ^ b) & kPg);
    }
    static int count(uint64_t) { return 1; }
    static uint64_t elem(uint64_t a, int) { return a; }
    static uint64_t ket(uint64_t a) { return a; }
    static uint64_t bra(uint64_t a, uint64_t dq) { return add(a, dq); }
    static uint64_t combine(uint64_t dq, uint64_t b, uint64_t k) {
        return add(k, dq) == b ? k : kInvalid;
    }
};

// ---- SU2LongLong: N (16, signed) | 2S_low (16) | 2S (16) | pg (16); a label
// from a sum carries the range 2S_low..2S of total spins (steps of 2)
struct Su2 {
    static uint64_t twos(uint64_t a) { return (a >> 16) & 0xFFFFULL; }
    static uint64_t neg(uint64_t a) {
        return (a & 0xFFFFFFFFFFFFULL) | ((~a + (1ULL << 48)) & kTop16);
    }
    static uint64_t add(uint64_t a, uint64_t b) {
        const uint64_t sum = (((a & kSumFields) + (b & kSumFields)) & kSumFields) | ((a ^ b) & kPg);
        // lowest coupled spin |S_a - S_b|: the difference that does not borrow
        const uint64_t d_ab = ((a & 0xFFFF0000ULL) << 16) - (b & 0xFFFF00000000ULL);
        const uint64_t d_ba = ((b & 0xFFFF0000ULL) << 16) - (a & 0xFFFF00000000ULL);
        return sum | std::min(d_ab, d_ba);
    }
    static int count(uint64_t a) { return (int)(((a >> 17) - (a >> 33)) & 0x7FFFULL) + 1; }
    static uint64_t elem(uint64_t a, int k) {
        const uint64_t x = a + ((uint64_t)k << 33);  // 2S_low + 2k
        return (x & 0xFFFFFFFF0000FFFFULL) | ((x & 0xFFFF00000000ULL) >> 16);
    }
    static uint64_t ket(uint64_t a) { return (a & 0xFFFF0000FFFFFFFFULL) | ((a & 0xFFFF0000ULL) << 16); }
    static uint64_t bra(uint64_t a, uint64_t dq) {
        return ((a & kTop16) + (dq & kTop16)) | ((a ^ dq) & kPg) | ((a & 0xFFFF00000000ULL) >> 16) |
               (a & 0xFFFF00000000ULL);
    }
    static bool triangle(int64_t ja, int64_t jb, int64_t jc) {
        return !((ja + jb + jc) & 1) && jc <= ja + jb && jc >= (ja > jb ? ja - jb : jb - ja);
    }
    static uint64_t combine(uint64_t dq, uint64_t b, uint64_t k) {
        k = (k & 0xFFFF0000FFFFFFFFULL) | (twos(b) << 32);  // ket's 2S_low := bra's 2S
        if (bra(k, dq) != b || !triangle((int64_t)twos(k), (int64_t)twos(dq), (int64_t)twos(b)))
            return kInvalid;
        return k;
    }
};

struct States {
    std::vector<uint64_t> q;
    std::vector<uint64_t> n;  // counts before saturation to the bond type
};

int find(const uint64_t *q, int n, uint64_t x) {
    const uint64_t *p = std::lower_bound(q, q + n, x);
    return (p == q + n || *p != x) ? -1 : (int)(p - q);
}

// sort by label, drop empty entries and labels above target, merge equal labels
// (counts saturate at ubond_max)
void sort_collect(States &s, uint64_t target, uint64_t ubond_max) {
    std::vector<size_t> idx(s.q.size());
    for (size_t i = 0; i < idx.size(); i++)
        idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(), [&](size_t x, size_t y) { return s.q[x] < s.q[y]; });
    States o;
    for (size_t t : idx) {
        if (s.n[t] == 0 || target < s.q[t])
            continue;
        if (!o.q.empty() && o.q.back() == s.q[t])
            o.n.back() = std::min(o.n.back() + s.n[t], ubond_max);
        else
            o.q.push_back(s.q[t]), o.n.push_back(s.n[t]);
    }
    s = o;
}

template <class L>
int tensor_product(const b2g_state_info *a, const b2g_state_info *b, const b2g_state_info *cref,
                   uint64_t target, uint64_t ubond_max, States &c) {
    c = States();
    if (cref != nullptr) {
        c.q.assign(cref->quanta, cref->quanta + cref->n);
        c.n.assign(cref->n, 0);
    }
    for (int i = 0; i < a->n; i++)
        for (int j = 0; j < b->n; j++) {
            const uint64_t qc = L::add(a->quanta[i], b->quanta[j]);
            const uint64_t prod = std::min((uint64_t)a->n_states[i] * (uint64_t)b->n_states[j], ubond_max);
            for (int k = 0; k < L::count(qc); k++) {
                const uint64_t qk = L::elem(qc, k);
                if (cref == nullptr) {
                    c.q.push_back(qk), c.n.push_back(prod);
                    continue;
                }
                const int ic = find(c.q.data(), (int)c.q.size(), qk);
                if (ic != -1)
                    c.n[ic] = std::min((uint64_t)a->n_states[i] * (uint64_t)b->n_states[j] + c.n[ic],
                                       ubond_max);
            }
        }
    sort_collect(c, cref == nullptr ? target : kInvalid, ubond_max);
    return B2G_OK;
}

template <class L>
int connection(const b2g_state_info *a, const b2g_state_info *b, const b2g_state_info *c,
               std::vector<uint32_t> &acc, std::vector<uint32_t> &ij) {
    std::map<uint64_t, std::vector<std::pair<uint32_t, uint32_t>>> mp;
    for (int i = 0; i < a->n; i++)
        for (int j = 0; j < b->n; j++) {
            const uint64_t qc = L::add(a->quanta[i], b->quanta[j]);
            for (int k = 0; k < L::count(qc); k++)
                mp[L::elem(qc, k)].push_back({(uint32_t)i, (uint32_t)j});
        }
    acc.assign(1, 0);
    ij.clear();
    for (int ic = 0; ic < c->n; ic++) {
        auto it = mp.find(c->quanta[ic]);
        if (it == mp.end())
            return fail(B2G_ERR_ARG, "b2g_state_connection: label " + std::to_string(ic) +
                                         " of c is not a product of a and b");
        for (auto &p : it->second)
            ij.push_back(p.first), ij.push_back(p.second);
        acc.push_back((uint32_t)(ij.size() / 2));
    }
    return B2G_OK;
}

template <class L>
int blocks(const b2g_state_info *bra, const b2g_state_info *ket, uint64_t dq, bool wfn,
           std::vector<uint64_t> &q, std::vector<uint32_t> &rows, std::vector<uint32_t> &cols) {
    q.clear();
    for (int i = 0; i < ket->n; i++) {
        const uint64_t qk = wfn ? L::neg(ket->quanta[i]) : ket->quanta[i];
        const uint64_t bs = L::add(dq, qk);
        for (int k = 0; k < L::count(bs); k++) {
            const uint64_t b = L::elem(bs, k);
            if (find(bra->quanta, bra->n, b) != -1)
                q.push_back(L::combine(dq, b, qk));
        }
    }
    std::sort(q.begin(), q.end());
    rows.resize(q.size()), cols.resize(q.size());
    for (size_t i = 0; i < q.size(); i++) {
        const uint64_t kq = wfn ? L::neg(L::ket(q[i])) : L::ket(q[i]);
        const int ik = find(ket->quanta, ket->n, kq), ib = find(bra->quanta, bra->n, L::bra(q[i], dq));
        if (q[i] == kInvalid || ik < 0 || ib < 0)
            return fail(B2G_ERR_ARG, "b2g_wfn_blocks: block label outside the symmetry range");
        cols[i] = ket->n_states[ik], rows[i] = bra->n_states[ib];
    }
    return B2G_OK;
}

// ---- SU(2) recoupling coefficients (spins given as 2j), in long double
struct Recoupling {
    long double fact[200];
    Recoupling() {
        fact[0] = 1.0L;
        for (int i = 1; i < 200; i++)
            fact[i] = fact[i - 1] * (long double)i;
    }
    static bool tri(int a, int b, int c) {
        return !((a + b + c) & 1) && c <= a + b && c >= (a > b ? a - b : b - a);
    }
    // triangle coefficient Delta(abc) = sqrt((a+b-c)! (a-b+c)! (-a+b+c)! / (a+b+c+1)!)
    long double delta(int a, int b, int c) const {
        return sqrtl(fact[(a + b - c) / 2] * fact[(a - b + c) / 2] * fact[(-a + b + c) / 2] /
                     fact[(a + b + c) / 2 + 1]);
    }
    // 6j symbol {a b c; d e f} by Racah's single-sum formula
    long double sixj(int a, int b, int c, int d, int e, int f) const {
        if (!tri(a, b, c) || !tri(a, e, f) || !tri(d, b, f) || !tri(d, e, c))
            return 0.0L;
        const int t1 = (a + b + c) / 2, t2 = (a + e + f) / 2, t3 = (d + b + f) / 2, t4 = (d + e + c) / 2;
        const int u1 = (a + b + d + e) / 2, u2 = (b + c + e + f) / 2, u3 = (a + c + d + f) / 2;
        const int lo = std::max(std::max(t1, t2), std::max(t3, t4)), hi = std::min(u1, std::min(u2, u3));
        long double sum = 0.0L;
        for (int t = lo; t <= hi; t++) {
            const long double term = fact[t + 1] / (fact[t - t1] * fact[t - t2] * fact[t - t3] * fact[t - t4] *
                                                    fact[u1 - t] * fact[u2 - t] * fact[u3 - t]);
            sum += (t & 1) ? -term : term;
        }
        return delta(a, b, c) * delta(a, e, f) * delta(d, b, f) * delta(d, e, c) * sum;
    }
    // 9j symbol {a b c; d e f; g h i} as sum_x (-1)^(2x) (2x+1) {a b c; f i x}
    // {d e f; b x h} {g h i; x a d} (Messiah, Quantum Mechanics, App. C)
    long double ninej(int a, int b, int c, int d, int e, int f, int g, int h, int i) const {
        if (!tri(a, b, c) || !tri(d, e, f) || !tri(g, h, i) || !tri(a, d, g) || !tri(b, e, h) ||
            !tri(c, f, i))
            return 0.0L;
        const int lo = std::max(std::abs(a - i), std::max(std::abs(d - h), std::abs(b - f)));
        const int hi = std::min(a + i, std::min(d + h, b + f));
        long double sum = 0.0L;
        for (int x = lo; x <= hi; x += 2) {
            const long double t = (long double)(x + 1) * sixj(a, b, c, f, i, x) * sixj(d, e, f, b, x, h) *
                                  sixj(g, h, i, x, a, d);
            sum += (x & 1) ? -t : t;
        }
        return sum;
    }
    // factor of an SU(2) operator block used transposed: delta spin d, row /
    // column spins l / r (the reference's sign and normalisation convention)
    static long double transpose(int d, int l, int r) {
        const long double sign = ((d + l - r) & 2) ? -1.0L : 1.0L;
        return sign * sqrtl((long double)(r + 1)) / sqrtl((long double)(l + 1));
    }
};

struct OpInfos {
    const b2g_op_infos *p;
    int find_info(uint64_t dq) const {  // exact delta quantum or -1
        return find(p->dq, p->n, dq);
    }
    int find_block(int info, uint64_t q) const {
        const int s = p->start[info], e = p->start[info + 1];
        const int k = find(p->quanta + s, e - s, q);
        return k;
    }
};

struct CEntry {
    double f;
    uint64_t iv;
    uint32_t ia, ib, ic;
};

// ConnectionInfo::initialize_wfn (src/core/sparse_matrix.hpp:163-292): for
// every sub-label k (conj type, label) and every bra block iv, the coupled
// (left op block ia, right op block ib, ket block ic) with their factor; the
// j-th entry found for each iv goes to round j, and rounds are emitted in
// order (so the first entry of every bra block comes first).
template <class L, bool kSu2>
int wfn_connection(uint64_t cdq, uint64_t vdq, uint64_t opdq, int n_sub, const int32_t *sub_conj,
                   const uint64_t *sub_q, const OpInfos &A, const OpInfos &B, int n_ket,
                   const uint64_t *ket_q, int n_bra, const uint64_t *bra_q, int32_t *n5,
                   std::vector<uint32_t> &idx, std::vector<CEntry> &out) {
    static const Recoupling rc;
    auto tw = [](uint64_t a) { return (int)((a >> 16) & 0xFFFFULL); };
    auto mult = [&](uint64_t a) { return kSu2 ? tw(a) + 1 : 1; };
    auto fermion = [](uint64_t a) { return ((a >> 48) & 1ULL) != 0; };
    for (int t = 0; t < 5; t++)
        n5[t] = -1;
    idx.assign(n_sub, 0);
    for (int k = 0; k < n_sub; k++) {
        const int ct = sub_conj[k];
        if (ct < 0 || ct > 3)
            return fail(B2G_ERR_ARG, "b2g_wfn_connection: conj type outside 0..3");
        if (n5[ct] == -1)
            n5[ct] = k;
        const bool cja = ct & 1, cjb = (ct & 2) != 0;
        idx[k] = (uint32_t)out.size();
        const uint64_t sq = sub_q[k];
        const uint64_t adq = cja ? L::neg(L::bra(sq, opdq)) : L::bra(sq, opdq);
        const uint64_t bdq = cjb ? L::ket(sq) : L::neg(L::ket(sq));
        const int ai = A.find_info(adq), bi = B.find_info(bdq);
        if (ai < 0 || bi < 0)
            return fail(B2G_ERR_ARG, "b2g_wfn_connection: no operator info for a sub-label");
        const bool bferm = B.p->fermion[bi] != 0;
        std::vector<std::vector<CEntry>> rounds;
        for (int iv = 0; iv < n_bra; iv++) {
            size_t ip = 0;
            const uint64_t lq = L::bra(bra_q[iv], vdq);
            const uint64_t rq = L::neg(L::ket(bra_q[iv]));
            const uint64_t rqs = cjb ? L::add(rq, bdq) : L::add(rq, L::neg(bdq));
            for (int r = 0; r < L::count(rqs); r++) {
                const uint64_t rqp = L::elem(rqs, r);
                const int ib = B.find_block(bi, cjb ? L::combine(bdq, rqp, rq) : L::combine(bdq, rq, rqp));
                if (ib < 0)
                    continue;
                const uint64_t lqs = L::add(cdq, L::neg(rqp));
                for (int l = 0; l < L::count(lqs); l++) {
                    const uint64_t lqp = L::elem(lqs, l);
                    const int ia = A.find_block(ai, cja ? L::combine(adq, lqp, lq) : L::combine(adq, lq, lqp));
                    const int ic = find(ket_q, n_ket, L::combine(cdq, lqp, L::neg(rqp)));
                    if (ia < 0 || ic < 0)
                        continue;
                    long double x = 1.0L;
                    if (kSu2) {
                        x = sqrtl((long double)mult(cdq) * mult(opdq) * mult(lq) * mult(rq)) *
                            rc.ninej(tw(lqp), tw(rqp), tw(cdq), tw(adq), tw(bdq), tw(opdq), tw(lq), tw(rq),
                                     tw(vdq));
                        if (cja)
                            x *= Recoupling::transpose(tw(adq), tw(lq), tw(lqp));
                        if (cjb)
                            x *= Recoupling::transpose(tw(bdq), tw(rq), tw(rqp));
                    }
                    double f = (double)x;
                    if (bferm && fermion(lqp))
                        f = -f;
                    if (std::fabs(f) >= 1e-20) {
                        if (rounds.size() <= ip)
                            rounds.emplace_back();
                        rounds[ip].push_back(CEntry{f, (uint64_t)iv, (uint32_t)ia, (uint32_t)ib, (uint32_t)ic});
                        ip++;
                    }
                }
            }
        }
        for (auto &rd : rounds)
            out.insert(out.end(), rd.begin(), rd.end());
    }
    n5[4] = n_sub;
    for (int t = 3; t >= 0; t--)
        if (n5[t] == -1)
            n5[t] = n5[t + 1];
    return B2G_OK;
}

bool bad_info(const b2g_state_info *s) {
    return s == nullptr || s->n < 0 || (s->n > 0 && (s->quanta == nullptr || s->n_states == nullptr));
}

} // namespace
} // namespace b2g

using namespace b2g;

extern "C" {

int b2g_quanta_op(int sym, int op, uint64_t a, uint64_t b, uint64_t c, uint64_t *out) {
    if (out == nullptr || (sym != B2G_SYM_SZ && sym != B2G_SYM_SU2))
        return fail(B2G_ERR_ARG, "b2g_quanta_op: null output or unknown symmetry");
    const bool su2 = sym == B2G_SYM_SU2;
    switch (op) {
    case B2G_QOP_ADD: *out = su2 ? Su2::add(a, b) : Sz::add(a, b); break;
    case B2G_QOP_NEG: *out = su2 ? Su2::neg(a) : Sz::neg(a); break;
    case B2G_QOP_COUNT: *out = (uint64_t)(su2 ? Su2::count(a) : Sz::count(a)); break;
    case B2G_QOP_ELEM: *out = su2 ? Su2::elem(a, (int)b) : Sz::elem(a, (int)b); break;
    case B2G_QOP_KET: *out = su2 ? Su2::ket(a) : Sz::ket(a); break;
    case B2G_QOP_BRA: *out = su2 ? Su2::bra(a, b) : Sz::bra(a, b); break;
    case B2G_QOP_COMBINE: *out = su2 ? Su2::combine(a, b, c) : Sz::combine(a, b, c); break;
    default: return fail(B2G_ERR_ARG, "b2g_quanta_op: unknown operation");
    }
    return B2G_OK;
}

int b2g_state_tensor_product(int sym, uint32_t ubond_max, const b2g_state_info *a,
                             const b2g_state_info *b, const b2g_state_info *cref, uint64_t target,
                             b2g_state_info *c) {
    if (bad_info(a) || bad_info(b) || (cref != nullptr && bad_info(cref)) || c == nullptr ||
        (sym != B2G_SYM_SZ && sym != B2G_SYM_SU2) || ubond_max == 0)
        return fail(B2G_ERR_ARG, "b2g_state_tensor_product: bad argument");
    States r;
    const int rc = sym == B2G_SYM_SU2 ? tensor_product<Su2>(a, b, cref, target, ubond_max, r)
                                      : tensor_product<Sz>(a, b, cref, target, ubond_max, r);
    if (rc != B2G_OK)
        return rc;
    const int cap = c->n;
    c->n = (int32_t)r.q.size();
    if ((int)r.q.size() > cap)
        return fail(B2G_ERR_ARG, "b2g_state_tensor_product: output capacity " + std::to_string(cap) +
                                     " below " + std::to_string(r.q.size()));
    for (size_t i = 0; i < r.q.size(); i++)
        c->quanta[i] = r.q[i], c->n_states[i] = (uint32_t)r.n[i];
    return B2G_OK;
}

int b2g_state_connection(int sym, const b2g_state_info *a, const b2g_state_info *b,
                         const b2g_state_info *c, uint32_t *acc, uint32_t *ij, int64_t cap,
                         int64_t *n_pairs) {
    if (bad_info(a) || bad_info(b) || bad_info(c) || acc == nullptr || n_pairs == nullptr ||
        (sym != B2G_SYM_SZ && sym != B2G_SYM_SU2))
        return fail(B2G_ERR_ARG, "b2g_state_connection: bad argument");
    std::vector<uint32_t> va, vij;
    const int rc = sym == B2G_SYM_SU2 ? connection<Su2>(a, b, c, va, vij) : connection<Sz>(a, b, c, va, vij);
    if (rc != B2G_OK)
        return rc;
    *n_pairs = (int64_t)(vij.size() / 2);
    if (*n_pairs > cap || (*n_pairs > 0 && ij == nullptr))
        return fail(B2G_ERR_ARG, "b2g_state_connection: pair capacity too small");
    std::copy(va.begin(), va.end(), acc);
    std::copy(vij.begin(), vij.end(), ij);
    return B2G_OK;
}

int b2g_wfn_blocks(int sym, const b2g_state_info *bra, const b2g_state_info *ket, uint64_t dq,
                   int wfn, uint32_t align, uint64_t *quanta, uint32_t *rows, uint32_t *cols,
                   uint32_t *shifts, int cap, int *n_blocks, uint32_t *total) {
    if (bad_info(bra) || bad_info(ket) || n_blocks == nullptr || total == nullptr || align == 0 ||
        (sym != B2G_SYM_SZ && sym != B2G_SYM_SU2))
        return fail(B2G_ERR_ARG, "b2g_wfn_blocks: bad argument");
    std::vector<uint64_t> q;
    std::vector<uint32_t> r, k;
    const int rc = sym == B2G_SYM_SU2 ? blocks<Su2>(bra, ket, dq, wfn != 0, q, r, k)
                                      : blocks<Sz>(bra, ket, dq, wfn != 0, q, r, k);
    if (rc != B2G_OK)
        return rc;
    *n_blocks = (int)q.size();
    if ((int)q.size() > cap || (!q.empty() && (quanta == nullptr || rows == nullptr ||
                                               cols == nullptr || shifts == nullptr)))
        return fail(B2G_ERR_ARG, "b2g_wfn_blocks: output capacity too small");
    // block offsets in 32-bit arithmetic, each block rounded up to align
    uint32_t off = 0;
    for (size_t i = 0; i < q.size(); i++) {
        quanta[i] = q[i], rows[i] = r[i], cols[i] = k[i], shifts[i] = off;
        const uint32_t x = r[i] * k[i];
        off = off + (x + align - 1) / align * align;
    }
    *total = off;
    return B2G_OK;
}

int b2g_wfn_connection(int sym, uint64_t cdq, uint64_t vdq, uint64_t opdq, int32_t n_sub,
                       const int32_t *sub_conj, const uint64_t *sub_q, const b2g_op_infos *left,
                       const b2g_op_infos *right, int32_t n_ket, const uint64_t *ket_q, int32_t n_bra,
                       const uint64_t *bra_q, int32_t *n5, uint32_t *idx, uint64_t *stride,
                       double *factor, uint32_t *ia, uint32_t *ib, uint32_t *ic, int64_t cap,
                       int64_t *nc) {
    auto bad_ops = [](const b2g_op_infos *o) {
        return o == nullptr || o->n < 0 ||
               (o->n > 0 && (o->dq == nullptr || o->fermion == nullptr || o->start == nullptr ||
                             (o->start[o->n] > 0 && o->quanta == nullptr)));
    };
    if ((sym != B2G_SYM_SZ && sym != B2G_SYM_SU2) || n_sub < 0 || (n_sub > 0 && (sub_conj == nullptr ||
        sub_q == nullptr)) || bad_ops(left) || bad_ops(right) || n_ket < 0 || n_bra < 0 ||
        (n_ket > 0 && ket_q == nullptr) || (n_bra > 0 && bra_q == nullptr) || n5 == nullptr ||
        nc == nullptr || (n_sub > 0 && idx == nullptr))
        return fail(B2G_ERR_ARG, "b2g_wfn_connection: bad argument");
    std::vector<uint32_t> vi;
    std::vector<CEntry> out;
    const OpInfos A{left}, B{right};
    const int rc = sym == B2G_SYM_SU2
                       ? wfn_connection<Su2, true>(cdq, vdq, opdq, n_sub, sub_conj, sub_q, A, B, n_ket, ket_q,
                                                   n_bra, bra_q, n5, vi, out)
                       : wfn_connection<Sz, false>(cdq, vdq, opdq, n_sub, sub_conj, sub_q, A, B, n_ket, ket_q,
                                                   n_bra, bra_q, n5, vi, out);
    if (rc != B2G_OK)
        return rc;
    *nc = (int64_t)out.size();
    if (*nc > cap || (*nc > 0 && (stride == nullptr || factor == nullptr || ia == nullptr ||
                                  ib == nullptr || ic == nullptr)))
        return fail(B2G_ERR_ARG, "b2g_wfn_connection: output capacity too small");
    std::copy(vi.begin(), vi.end(), idx);
    for (size_t j = 0; j < out.size(); j++)
        stride[j] = out[j].iv, factor[j] = out[j].f, ia[j] = out[j].ia, ib[j] = out[j].ib, ic[j] = out[j].ic;
    return B2G_OK;
}

} // extern "C"
