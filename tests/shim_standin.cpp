// CPU stand-in for the C-ABI calls the shim makes when block2's own Davidson drives
// GpuTensorFunctions (operator(), the perturbative-noise product, the PDM expectation):
// contexts hold a host staging buffer and b2g_heff_apply_host replays the recorded pairs with
// the oracle (oracle/b2g_oracle.c), so the shim's host-side translation of block2's
// products into pairs runs, and is checked, without a GPU.  Test infrastructure only.
#include <cstring>
#include <string>
#include <vector>
#include "b2g.h"
extern "C" int b2g_oracle_replay(const b2g_pair_seq *s, const double *ops, const double *psi, double *sigma,
                                 uint64_t sigma_size, double scale, int nthreads);
struct b2g_context {
    int dev;
    std::vector<double> stage;  // b2g_host_buffer
};
struct b2g_heff {
    std::vector<int32_t> i[12]; std::vector<double> f[2]; std::vector<uint64_t> u[4];
    b2g_pair_seq s; std::vector<double> ops; uint64_t np, ns;
};
static std::string err;
// the library's error channel, used by the host-only translator linked in
// (b2g_noise_pairs, block2-preview_gb300/csrc/b2g_noise.cu)
namespace b2g {
int fail(int code, const std::string &msg) {
    err = msg;
    return code;
}
} // namespace b2g
extern "C" {
// device-only entries of GpuDMRG: not on the paths this stand-in serves
int b2g_heff_diag_host(b2g_heff *, double *) { return b2g::fail(B2G_ERR_UNSUPPORTED, "stand-in"); }
int b2g_davidson(b2g_heff *, const double *, double *, double, int, int, int, int, b2g_davidson_result *) {
    return b2g::fail(B2G_ERR_UNSUPPORTED, "stand-in");
}
int b2g_davidson_multi(b2g_heff *, const double *, double *, int, double, int, int, int, int, double *,
                       b2g_davidson_result *) {
    return b2g::fail(B2G_ERR_UNSUPPORTED, "stand-in");
}
int b2g_context_create(int device, b2g_context **out) {
    *out = new b2g_context();
    (*out)->dev = device;
    return 0;
}
int b2g_host_buffer(b2g_context *c, uint64_t bytes, void **out) {
    if (c->stage.size() * 8 < bytes)
        c->stage.assign((bytes + 7) / 8, 0.0);
    *out = c->stage.data();
    return 0;
}
int b2g_heff_set_ops(b2g_heff *h, const double *ops, int) {
    std::memcpy(h->ops.data(), ops, sizeof(double) * h->ops.size());
    return 0;
}
int b2g_context_destroy(b2g_context *c) { delete c; return 0; }
const char *b2g_last_error(void) { return err.c_str(); }
int b2g_launch_count(uint64_t *o) { *o = 0; return 0; }
int b2g_heff_create(b2g_context *, const b2g_pair_seq *s, const double *ops, uint64_t ops_size, int,
                    uint64_t np, uint64_t ns, b2g_heff **out) {
    auto *h = new b2g_heff();
    const int32_t *ip[12] = {s->tb0, s->m0, s->n0, s->k0, s->lda0, s->ldb0, s->ta1, s->m1, s->n1, s->k1, s->lda1, s->ldc1};
    for (int q = 0; q < 12; q++) h->i[q].assign(ip[q], ip[q] + s->n_pairs);
    h->f[0].assign(s->alpha0, s->alpha0 + s->n_pairs), h->f[1].assign(s->alpha1, s->alpha1 + s->n_pairs);
    const uint64_t *up[4] = {s->a0, s->b0, s->a1, s->c1};
    for (int q = 0; q < 4; q++) h->u[q].assign(up[q], up[q] + s->n_pairs);
    h->s.n_pairs = s->n_pairs;
    h->s.tb0 = h->i[0].data(), h->s.m0 = h->i[1].data(), h->s.n0 = h->i[2].data(), h->s.k0 = h->i[3].data();
    h->s.lda0 = h->i[4].data(), h->s.ldb0 = h->i[5].data(), h->s.ta1 = h->i[6].data(), h->s.m1 = h->i[7].data();
    h->s.n1 = h->i[8].data(), h->s.k1 = h->i[9].data(), h->s.lda1 = h->i[10].data(), h->s.ldc1 = h->i[11].data();
    h->s.alpha0 = h->f[0].data(), h->s.alpha1 = h->f[1].data();
    h->s.a0 = h->u[0].data(), h->s.b0 = h->u[1].data(), h->s.a1 = h->u[2].data(), h->s.c1 = h->u[3].data();
    if (ops != nullptr)
        h->ops.assign(ops, ops + ops_size);
    else
        h->ops.assign(ops_size, 0.0);  // B2G_OPS_DEFERRED: filled by b2g_heff_set_ops
    h->np = np, h->ns = ns;
    *out = h; return 0;
}
int b2g_heff_destroy(b2g_heff *h) { delete h; return 0; }
int b2g_heff_apply_host(b2g_heff *h, const double *psi, double *sigma, double scale, int) {
    return b2g_oracle_replay(&h->s, h->ops.data(), psi, sigma, h->ns, scale, 1);
}
}
