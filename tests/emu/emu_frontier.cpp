/* Runs k_frontier (BFS or SSSP, optional bottom-up rounds or light/heavy
 * classes) on NB emulated blocks and compares with the oracle's distances.
 * args: dir NB row sssp iters delta bu alpha beta lh [pull [tail]]
 * (pull: bucket closes by pull, 0 never, 1 cost rule, 2 always; the test
 * graphs have equal weights both ways; tail: buckets end once one opens
 * with at most this many far-pile entries, 0 never) */
#include "kernel_frontier.inc"
template <int BS, bool SSSP>
int run(int NB, const std::string &d, int row, uint32_t iters, uint32_t bu, uint32_t alpha, uint32_t beta,
        uint32_t delta, bool lhm, uint32_t pull, uint32_t tail) {
    auto off = rd(d + "/off.bin"), col = rd(d + "/col.bin"), wt = rd(d + "/wt.bin"), srcs = rd(d + "/srcs.bin");
    auto want = rd(d + (SSSP ? "/want_sssp.bin" : "/want_bfs.bin"));
    uint32_t n = off.size() - 1, m = col.size(), src = srcs[row];
    uint32_t cap = std::max<uint32_t>(1024, n), ucap = m / 512 + 4;
    std::vector<uint32_t> dist(cap), bits(cap / 32 + 2), farbits(cap / 32 + 2), stamp(cap), q[6], uf[2], far[3];
    for (auto &x : q) x.assign(cap, 0);
    for (auto &x : uf) x.assign(ucap, 0);
    for (auto &x : far) x.assign(cap, 0);
    FrontierCtl ctl;
    memset(&ctl, 0, sizeof ctl);
    Args a;
    memset(&a, 0, sizeof a);
    a.off = off.data(); a.col = col.data(); a.wt = wt.data(); a.n = n; a.m = m;
    a.dist = dist.data(); a.bits = bits.data(); a.farbits = farbits.data(); a.stamp = stamp.data();
    a.qv0 = q[0].data(); a.qv1 = q[1].data(); a.qo0 = q[2].data(); a.qo1 = q[3].data(); a.qb0 = q[4].data(); a.qb1 = q[5].data();
    a.uf0 = uf[0].data(); a.uf1 = uf[1].data(); a.far0 = far[0].data(); a.far1 = far[1].data(); a.far2 = far[2].data();
    a.ctl = &ctl; a.cap = cap; a.ucap = ucap; a.src = src; a.iters = iters; a.unit = BS * iters; a.scap = BS * 9;
    a.delta = delta; a.nblocks = NB; a.max_rounds = 4 * n + 4096; a.timeout_ns = 60000000000ull;
    a.bu = bu; a.alpha = alpha; a.beta = beta;
    if (SSSP && delta) a.tail_at = tail;
    std::vector<uint32_t> lcol(m + 4), lwt(m + 4), light(n + 1), hstamp(cap), pbest(cap), hq[9], huf[3];
    for (auto &x : hq) x.assign(cap, 0);
    for (auto &x : huf) x.assign(ucap, 0);
    if (SSSP && delta && lhm) { /* light-first, class-ordered rows, as dev_graph_light_heavy builds them */
        uint32_t maxw = 0;
        for (uint32_t e = 0; e < m; ++e) maxw = std::max(maxw, wt[e]);
        const uint32_t cw = maxw >= delta ? (maxw - delta + LH_CLASSES) / LH_CLASSES : 1;
        auto cls = [&](uint32_t w) { return w < delta ? 0u : 1u + std::min((w - delta) / cw, LH_CLASSES - 1); };
        for (uint32_t u = 0; u < n; ++u) {
            uint32_t p = off[u];
            for (uint32_t c = 0; c <= LH_CLASSES; ++c)
                for (uint32_t e = off[u]; e < off[u + 1]; ++e)
                    if (cls(wt[e]) == c) { lcol[p] = col[e]; lwt[p] = wt[e]; ++p; }
            light[u] = 0;
            for (uint32_t e = off[u]; e < off[u + 1]; ++e) light[u] += wt[e] < delta;
        }
        a.cw = cw;
        a.col = lcol.data(); a.wt = lwt.data(); a.light = light.data(); a.hstamp = hstamp.data();
        a.hv0 = hq[0].data(); a.hv1 = hq[1].data(); a.hv2 = hq[2].data();
        a.ho0 = hq[3].data(); a.ho1 = hq[4].data(); a.ho2 = hq[5].data();
        a.hb0 = hq[6].data(); a.hb1 = hq[7].data(); a.hb2 = hq[8].data();
        a.huf0 = huf[0].data(); a.huf1 = huf[1].data(); a.huf2 = huf[2].data();
        a.pull = pull;
        a.pbest = pbest.data();
        for (uint32_t e = 0; e < m; ++e) a.heavy_edges += wt[e] >= delta;
    }
    run_grid(NB, BS, [&](int b) {
        switch (b) {
        case 0: k_frontier<BS, SSSP, 0>(a); break;
        case 1: k_frontier<BS, SSSP, 1>(a); break;
        case 2: k_frontier<BS, SSSP, 2>(a); break;
        default: k_frontier<BS, SSSP, 3>(a);
        }
    });
    size_t bad = 0;
    for (uint32_t i = 0; i < n; ++i) bad += dist[i] != want[(size_t)row * n + i];
    printf("frontier sssp=%d lh=%d pull=%u row=%d iters=%u delta=%u bu=%u err=%u rounds=%u bad=%zu relaxed=%llu\n",
           (int)SSSP, a.light != nullptr, a.pull, row, iters, delta, bu, ctl.err, ctl.rounds, bad, ctl.edges_relaxed);
    return bad != 0 || ctl.err;
}
int main(int argc, char **argv) {
    if (argc < 11) return 3;
    std::string d = argv[1];
    int nb = atoi(argv[2]), row = atoi(argv[3]), sssp = atoi(argv[4]);
    uint32_t iters = atoi(argv[5]), delta = atoi(argv[6]), bu = atoi(argv[7]), al = atoi(argv[8]), be = atoi(argv[9]);
    bool lhm = atoi(argv[10]);
    uint32_t pull = argc > 11 ? atoi(argv[11]) : 0, tail = argc > 12 ? atoi(argv[12]) : 0;
    return sssp ? run<256, true>(nb, d, row, iters, 0, al, be, delta, lhm, pull, tail)
                : run<256, false>(nb, d, row, iters, bu, al, be, 0, false, 0, 0);
}
