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
//     (src/core/sparse_matrix.hpp:617-630, 727-757, 804-820).
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

} // extern "C"
