/* Runs k_msbfs for the first nsrc sources.  args: dir NB nsrc [bu]
 * (bu: bottom-up levels allowed; the test graphs are symmetric) */
#include "kernel_msbfs.inc"
int main(int argc, char **argv) {
    if (argc < 4) return 3;
    std::string d = argv[1];
    int NB = atoi(argv[2]);
    uint32_t nsrc = atoi(argv[3]);
    auto off = rd(d + "/off.bin"), col = rd(d + "/col.bin"), srcs = rd(d + "/srcs.bin"), want = rd(d + "/want_bfs.bin");
    uint32_t n = off.size() - 1, m = col.size(), ucap = m / MB_UNIT + 4;
    std::vector<unsigned long long> seen(n), nxt(n), xf(n);
    std::vector<uint32_t> cand(n), xv(n), xo(n), xb(n), uf(ucap), dist((size_t)nsrc * n, 1000000000u);
    MsCtl ctl;
    memset(&ctl, 0, sizeof ctl);
    MsArgs a;
    memset(&a, 0, sizeof a);
    a.off = off.data(); a.col = col.data(); a.n = n; a.m = m; a.seen = seen.data(); a.nxt = nxt.data();
    a.cand = cand.data(); a.xv = xv.data(); a.xo = xo.data(); a.xb = xb.data(); a.xf = xf.data(); a.uf = uf.data();
    a.dist = dist.data(); a.ns = nsrc; a.ctl = &ctl; a.ucap = ucap; a.nblocks = NB; a.max_levels = n + 1;
    a.timeout_ns = 60000000000ull;
    a.bu = argc > 4 ? atoi(argv[4]) : 0;
    a.all = nsrc == 64 ? ~0ull : (1ull << nsrc) - 1;
    for (uint32_t s = 0; s < nsrc; ++s) { /* k_ms_sources */
        const uint32_t v = srcs[s];
        if (atomicOr(a.nxt + v, 1ull << s) == 0) a.cand[ctl.cand[0]++] = v;
    }
    run_grid(NB, MB_BS, [&](int b) {
        switch (b) { case 0: k_msbfs<0>(a); break; case 1: k_msbfs<1>(a); break; case 2: k_msbfs<2>(a); break; default: k_msbfs<3>(a); }
    });
    size_t bad = 0;
    for (uint32_t s = 0; s < nsrc; ++s)
        for (uint32_t v = 0; v < n; ++v) bad += dist[(size_t)v * nsrc + s] != want[(size_t)s * n + v];
    printf("msbfs NB=%d nsrc=%u bu=%u err=%u levels=%u bad=%zu relaxed=%llu\n", NB, nsrc, a.bu, ctl.err, ctl.levels, bad,
           ctl.edges_relaxed);
    return bad != 0 || ctl.err;
}
