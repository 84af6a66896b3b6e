// Term partition of one H_eff over several ranks (host only).
//
// The reference distributes the H_eff terms over MPI ranks by operator site
// indices (ParallelRuleQC, src/dmrg/qc_parallel_rule.hpp:31-85); each rank
// replays its own BatchGEMMSeq and the partial sigmas are summed with
// allreduce_sum (ParallelTensorFunctions::operator(),
// src/core/parallel_tensor_functions.hpp:51-55).  Here the unit of work is the
// recorded GEMM pair.  Pairs that share a GEMM0 product (same psi sub-block,
// same right operator block) must stay on one rank, or the product would be
// computed once per rank; every such group is one indivisible job.  Jobs are
// assigned largest first to the least-loaded rank (longest-processing-time
// rule), ties to the lower rank and to the earlier job, so every rank derives
// the same partition from the same sequence with no communication.
#include <algorithm>
#include <string>
#include <unordered_map>
#include <vector>

#include "b2g_internal.h"

namespace b2g {
namespace {

struct ProductKey {
    uint64_t a0, b0;
    int32_t m0, n0, k0, lda0, ldb0, tb0;
    bool operator==(const ProductKey &o) const {
        return a0 == o.a0 && b0 == o.b0 && m0 == o.m0 && n0 == o.n0 && k0 == o.k0 &&
               lda0 == o.lda0 && ldb0 == o.ldb0 && tb0 == o.tb0;
    }
};
struct ProductKeyHash {
    size_t operator()(const ProductKey &k) const {
        uint64_t h = k.a0 * 0x9E3779B97F4A7C15ULL ^ (k.b0 + 0x632BE59BD9B4E019ULL);
        h ^= ((uint64_t)(uint32_t)k.m0 << 32 | (uint32_t)k.n0) * 0xBF58476D1CE4E5B9ULL;
        h ^= ((uint64_t)(uint32_t)k.k0 << 32 | (uint32_t)k.lda0) * 0x94D049BB133111EBULL;
        h ^= ((uint64_t)(uint32_t)k.ldb0 << 1 | (uint32_t)k.tb0) * 0xD6E8FEB86659FD93ULL;
        return (size_t)(h ^ (h >> 31));
    }
};

} // namespace
} // namespace b2g

using namespace b2g;

extern "C" int b2g_partition_pairs(const b2g_pair_seq *seq, int n_ranks, int32_t *rank_of_pair,
                                   double *load) {
    if (seq == nullptr || n_ranks < 1 || seq->n_pairs < 0 ||
        (seq->n_pairs > 0 && rank_of_pair == nullptr))
        return fail(B2G_ERR_ARG, "b2g_partition_pairs: null argument or n_ranks < 1");
    const int64_t np = seq->n_pairs;
    // jobs: one per distinct GEMM0 product, in order of first appearance
    std::unordered_map<ProductKey, int64_t, ProductKeyHash> jmap;
    jmap.reserve((size_t)np * 2 + 1);
    std::vector<int64_t> job_of(np);
    std::vector<double> cost;
    for (int64_t i = 0; i < np; i++) {
        const int32_t m0 = seq->m0[i], n0 = seq->n0[i], k0 = seq->k0[i];
        const int32_t m1 = seq->m1[i], n1 = seq->n1[i], k1 = seq->k1[i];
        if (m0 < 0 || n0 < 0 || k0 < 0 || m1 < 0 || n1 < 0 || k1 < 0)
            return fail(B2G_ERR_ARG, "b2g_partition_pairs: pair " + std::to_string(i) +
                                         " has a negative dimension");
        const ProductKey key{seq->a0[i], seq->b0[i], m0, n0, k0, seq->lda0[i], seq->ldb0[i],
                             seq->tb0[i] ? 1 : 0};
        auto it = jmap.find(key);
        int64_t j;
        if (it == jmap.end()) {
            j = (int64_t)cost.size();
            jmap.emplace(key, j);
            cost.push_back((double)m0 * n0 * k0);  // the product, computed once
        } else
            j = it->second;
        job_of[i] = j;
        cost[j] += (double)m1 * n1 * k1;
    }
    const int64_t nj = (int64_t)cost.size();
    std::vector<int64_t> order(nj);
    for (int64_t j = 0; j < nj; j++)
        order[j] = j;
    std::stable_sort(order.begin(), order.end(),
                     [&](int64_t a, int64_t b) { return cost[a] > cost[b]; });
    std::vector<double> ld(n_ranks, 0.0);
    std::vector<int32_t> rank_of_job(nj, 0);
    for (int64_t j : order) {
        int32_t best = 0;
        for (int32_t r = 1; r < n_ranks; r++)
            if (ld[r] < ld[best])
                best = r;
        rank_of_job[j] = best;
        ld[best] += cost[j];
    }
    for (int64_t i = 0; i < np; i++)
        rank_of_pair[i] = rank_of_job[job_of[i]];
    if (load != nullptr)
        for (int32_t r = 0; r < n_ranks; r++)
            load[r] = ld[r];
    return B2G_OK;
}
