/* Runs k_sssp32 for the first nsrc sources.  args: dir NB nsrc */
#include "kernel_sssp32.inc"
int main(int argc, char **argv) {
    if (argc < 4) return 3;
    std::string d = argv[1];
    int NB = atoi(argv[2]);
    uint32_t nsrc = atoi(argv[3]);
    auto off = rd(d + "/off.bin"), col = rd(d + "/col.bin"), wt = rd(d + "/wt.bin"), srcs = rd(d + "/srcs.bin");
    auto want = rd(d + "/want_sssp.bin");
    uint32_t n = off.size() - 1, m = col.size(), ucap = m / SU_UNIT + 4;
    std::vector<uint32_t> D((size_t)n * 32, 1000000000u), M[3], qv[3], qo[2], qb[2], uf[2];
    for (auto &x : M) x.assign(n, 0);
    for (auto &x : qv) x.assign(n, 0);
    for (auto &x : qo) x.assign(n, 0);
    for (auto &x : qb) x.assign(n, 0);
    for (auto &x : uf) x.assign(ucap, 0);
    SuCtl ctl;
    memset(&ctl, 0, sizeof ctl);
    SuArgs a;
    memset(&a, 0, sizeof a);
    a.off = off.data(); a.col = col.data(); a.wt = wt.data(); a.n = n; a.m = m; a.D = D.data();
    a.M0 = M[0].data(); a.M1 = M[1].data(); a.M2 = M[2].data();
    a.qv0 = qv[0].data(); a.qv1 = qv[1].data(); a.qv2 = qv[2].data();
    a.qo0 = qo[0].data(); a.qo1 = qo[1].data(); a.qb0 = qb[0].data(); a.qb1 = qb[1].data();
    a.uf0 = uf[0].data(); a.uf1 = uf[1].data();
    a.ctl = &ctl; a.ucap = ucap; a.nblocks = NB; a.max_rounds = n + 2; a.timeout_ns = 60000000000ull;
    for (uint32_t s = 0; s < nsrc; ++s) { /* k_su_sources */
        const uint32_t v = srcs[s];
        D[(size_t)v * 32 + s] = 0;
        if (atomicOr(a.M0 + v, 1u << s) == 0) {
            const uint32_t b = off[v], dd = off[v + 1] - b;
            if (!dd) continue;
            const unsigned long long old = atomicAdd(&ctl.qctr[0], (1ull << 32) | dd);
            const uint32_t i = old >> 32, o = (uint32_t)old;
            a.qv0[i] = v; a.qo0[i] = o; a.qb0[i] = b;
            for (uint64_t k = (o + SU_UNIT - 1) / SU_UNIT; k * SU_UNIT < (uint64_t)o + dd; ++k) a.uf0[k] = i;
        }
    }
    run_grid(NB, SU_BS, [&](int b) {
        switch (b) { case 0: k_sssp32<0>(a); break; case 1: k_sssp32<1>(a); break; case 2: k_sssp32<2>(a); break; default: k_sssp32<3>(a); }
    });
    size_t bad = 0;
    for (uint32_t s = 0; s < nsrc; ++s)
        for (uint32_t v = 0; v < n; ++v) bad += D[(size_t)v * 32 + s] != want[(size_t)s * n + v];
    printf("sssp32 NB=%d nsrc=%u err=%u rounds=%u bad=%zu relaxed=%llu\n", NB, nsrc, ctl.err, ctl.rounds, bad, ctl.edges_relaxed);
    return bad != 0 || ctl.err;
}
