/* Drives k_mq the way the server does: supersteps of `per` rounds, `stagger`
 * new queries injected before each (0 = all at once), finished queries
 * detected by their queue entries and far-pile items (k_mq_count).
 * Queries: the first 16 sources of srcs.bin, algorithm from algos.bin, SSSP
 * bucket width `delta` (0 = Bellman-Ford order).  args: dir NB per stagger delta [tail [sof]]
 * (tail: a query's buckets end once its pile is at most this size and
 * shrinking; 0 never; sof: 1 = the server's supersteps, which also stop at the
 * first round in which a query finished and count each slot's remaining
 * work in the launch, checked against the k_mq_count figures; 2..15: the
 * same, stopping once that many finished; sof >= 16: the server's flow with
 * sof - 16 slots, reused as queries retire, stopping once half of the
 * queries in flight finished) */
#include "kernel_mq.inc"
int NB;
void launch(MqArgs a) {
    memset(&a.ctl->bar, 0, sizeof(GridBarrier));
    run_grid(NB, MQ_BS, [&](int b) {
        switch (b) { case 0: k_mq<0>(a); break; case 1: k_mq<1>(a); break; case 2: k_mq<2>(a); break; default: k_mq<3>(a); }
    });
}
/* The server's flow: `nslot` table slots, queries admitted into free slots
 * (a retired query's slot is reused), supersteps that stop at the first
 * finished query and count each slot's remaining work in the launch; a
 * query's distances are taken when its slot retires. */
int run_server(const std::string &d, uint32_t nslot, uint32_t per, uint32_t delta, uint32_t tail) {
    auto off = rd(d + "/off.bin"), col = rd(d + "/col.bin"), wt = rd(d + "/wt.bin"), srcs = rd(d + "/srcs.bin"),
         algos = rd(d + "/algos.bin"), want = rd(d + "/want_mix.bin");
    const uint32_t n = off.size() - 1, m = col.size(), nq = algos.size();
    const uint32_t cap = n * nslot, ucap = (uint32_t)((uint64_t)m * nslot / MQ_UNIT + 4);
    std::vector<uint32_t> q[8], uf[2];
    for (auto &x : q) x.assign(cap, 0);
    for (auto &x : uf) x.assign(ucap, 0);
    std::vector<std::vector<uint32_t>> dist(nslot, std::vector<uint32_t>(n)), aux(nslot, std::vector<uint32_t>(n)),
        fb(nslot, std::vector<uint32_t>(n / 32 + 1)), p0(nslot, std::vector<uint32_t>(n)), p1(nslot, std::vector<uint32_t>(n));
    std::vector<MqQuery> qt(nslot);
    std::vector<MqQstate> qs(nslot);
    memset(qt.data(), 0, nslot * sizeof(MqQuery));
    memset(qs.data(), 0, nslot * sizeof(MqQstate));
    MqCtl ctl;
    memset(&ctl, 0, sizeof ctl);
    MqArgs a;
    memset(&a, 0, sizeof a);
    a.qt = qt.data(); a.qs = qs.data(); a.nq = nslot; a.nearfar = nslot <= MQ_MAXQ;
    a.qq0 = q[0].data(); a.qq1 = q[1].data(); a.qv0 = q[2].data(); a.qv1 = q[3].data();
    a.qo0 = q[4].data(); a.qo1 = q[5].data(); a.qb0 = q[6].data(); a.qb1 = q[7].data();
    a.uf0 = uf[0].data(); a.uf1 = uf[1].data();
    a.ctl = &ctl; a.cap = cap; a.ucap = ucap; a.nblocks = NB; a.timeout_ns = 60000000000ull;
    std::vector<uint32_t> kact(nslot, 0);
    a.active = kact.data();
    std::vector<int> slot_q(nslot, -1);
    uint32_t next = 0, done_q = 0, launches = 0;
    size_t bad = 0;
    while (done_q < nq) {
        std::vector<uint32_t> list;
        for (uint32_t sl = 0; sl < nslot && next < nq; ++sl) {
            if (slot_q[sl] >= 0) continue;
            const uint32_t t = next++;
            slot_q[sl] = (int)t;
            MqQuery &Q = qt[sl]; /* k_mq_init */
            memset(&Q, 0, sizeof Q);
            Q.off = off.data(); Q.col = col.data(); Q.wt = wt.data(); Q.n = n; Q.m = m;
            Q.algo = algos[t]; Q.src = srcs[t]; Q.delta = Q.algo == GGA_SSSP ? delta : 0;
            Q.tail_at = Q.delta ? tail : 0;
            Q.dist = dist[sl].data(); Q.aux = aux[sl].data();
            Q.fbits = fb[sl].data(); Q.pile0 = p0[sl].data(); Q.pile1 = p1[sl].data();
            std::fill(dist[sl].begin(), dist[sl].end(), 1000000000u);
            std::fill(aux[sl].begin(), aux[sl].end(), 0u);
            std::fill(fb[sl].begin(), fb[sl].end(), 0u);
            list.push_back(sl);
        }
        threadIdx.x = 0;
        blockIdx.x = 0;
        if (!list.empty()) k_mq_inject(a, qt.data(), list.data(), list.size());
        a.max_rounds = per;
        uint32_t busy = 0;
        for (uint32_t sl = 0; sl < nslot; ++sl) busy += slot_q[sl] >= 0;
        a.stop_on_finish = std::max<uint32_t>(1u, busy / 2); /* as the server: a share of the queries in flight */
        std::fill(kact.begin(), kact.end(), 0u);
        launch(a);
        launches++;
        if (ctl.err) { printf("mq err=%u\n", ctl.err); return 1; }
        for (uint32_t sl = 0; sl < nslot; ++sl) { /* retire */
            if (slot_q[sl] < 0 || kact[sl] != 0) continue;
            const uint32_t t = (uint32_t)slot_q[sl];
            for (uint32_t v = 0; v < n; ++v) bad += dist[sl][v] != want[(size_t)t * n + v];
            slot_q[sl] = -1;
            done_q++;
        }
        if (launches > 100000) { printf("mq no progress\n"); return 1; }
    }
    printf("mq server delta=%u NB=%d slots=%u per=%u launches=%u rounds=%u err=%u bad=%zu relaxed=%llu\n", delta, NB,
           nslot, per, launches, ctl.rounds_done, ctl.err, bad, ctl.edges_relaxed);
    return bad != 0;
}
int main(int argc, char **argv) {
    if (argc < 6) return 3;
    std::string d = argv[1];
    NB = atoi(argv[2]);
    const uint32_t per = atoi(argv[3]), stagger = atoi(argv[4]), delta = atoi(argv[5]);
    const uint32_t tail = argc > 6 ? atoi(argv[6]) : 0, sof = argc > 7 ? atoi(argv[7]) : 0;
    if (sof >= 16) return run_server(d, sof - 16, per, delta, tail); /* sof - 16 = slots of the server flow */
    auto off = rd(d + "/off.bin"), col = rd(d + "/col.bin"), wt = rd(d + "/wt.bin"), srcs = rd(d + "/srcs.bin"),
         algos = rd(d + "/algos.bin"), want = rd(d + "/want_mix.bin");
    const uint32_t n = off.size() - 1, m = col.size(), nq = algos.size();
    const uint32_t cap = n * nq, ucap = (uint32_t)((uint64_t)m * nq / MQ_UNIT + 4);
    std::vector<uint32_t> q[8], uf[2];
    for (auto &x : q) x.assign(cap, 0);
    for (auto &x : uf) x.assign(ucap, 0);
    std::vector<std::vector<uint32_t>> dist(nq, std::vector<uint32_t>(n)), aux(nq, std::vector<uint32_t>(n)),
        fb(nq, std::vector<uint32_t>(n / 32 + 1)), p0(nq, std::vector<uint32_t>(n)), p1(nq, std::vector<uint32_t>(n));
    std::vector<MqQuery> qt(nq);
    std::vector<MqQstate> qs(nq);
    memset(qt.data(), 0, nq * sizeof(MqQuery));
    memset(qs.data(), 0, nq * sizeof(MqQstate));
    MqCtl ctl;
    memset(&ctl, 0, sizeof ctl);
    MqArgs a;
    memset(&a, 0, sizeof a);
    a.qt = qt.data(); a.qs = qs.data(); a.nq = nq; a.nearfar = nq <= MQ_MAXQ;
    a.qq0 = q[0].data(); a.qq1 = q[1].data(); a.qv0 = q[2].data(); a.qv1 = q[3].data();
    a.qo0 = q[4].data(); a.qo1 = q[5].data(); a.qb0 = q[6].data(); a.qb1 = q[7].data();
    a.uf0 = uf[0].data(); a.uf1 = uf[1].data();
    a.ctl = &ctl; a.cap = cap; a.ucap = ucap; a.nblocks = NB; a.timeout_ns = 60000000000ull;
    std::vector<int> admitted(nq, 0), finished(nq, 0);
    std::vector<uint32_t> kact(nq, 0);
    if (sof) {
        a.stop_on_finish = sof;
        a.active = kact.data();
    }
    uint32_t next = 0, launches = 0;
    for (;;) {
        std::vector<uint32_t> list;
        while (next < nq && (stagger == 0 || list.size() < stagger)) list.push_back(next++);
        for (uint32_t t : list) { /* k_mq_init */
            MqQuery &Q = qt[t];
            memset(&Q, 0, sizeof Q);
            Q.off = off.data(); Q.col = col.data(); Q.wt = wt.data(); Q.n = n; Q.m = m;
            Q.algo = algos[t]; Q.src = srcs[t]; Q.delta = Q.algo == GGA_SSSP ? delta : 0;
            Q.tail_at = Q.delta ? tail : 0;
            Q.dist = dist[t].data(); Q.aux = aux[t].data();
            Q.fbits = fb[t].data(); Q.pile0 = p0[t].data(); Q.pile1 = p1[t].data();
            std::fill(dist[t].begin(), dist[t].end(), 1000000000u);
            std::fill(aux[t].begin(), aux[t].end(), 0u);
            std::fill(fb[t].begin(), fb[t].end(), 0u);
            admitted[t] = 1;
        }
        threadIdx.x = 0;
        blockIdx.x = 0;
        if (!list.empty()) k_mq_inject(a, qt.data(), list.data(), list.size());
        a.max_rounds = per;
        std::fill(kact.begin(), kact.end(), 0u);
        launch(a);
        launches++;
        if (ctl.err) { printf("mq err=%u\n", ctl.err); return 1; }
        std::vector<uint32_t> active(nq, 0); /* k_mq_count */
        {
            const uint32_t r = ctl.round;
            const unsigned long long qc = ctl.qctr[r % 3];
            const uint32_t ni = std::min<uint32_t>(qc >> 32, cap);
            const uint32_t *qq = (r & 1) ? a.qq1 : a.qq0;
            for (uint32_t i = 0; i < ni; ++i) active[qq[i]]++;
            for (uint32_t t = 0; t < nq; ++t) active[t] += qs[t].fc[qs[t].fp[r & 1] & 1];
        }
        if (sof)
            for (uint32_t t = 0; t < nq; ++t)
                if (kact[t] != active[t]) {
                    printf("mq active mismatch slot %u kernel %u count %u\n", t, kact[t], active[t]);
                    return 1;
                }
        uint32_t live = 0;
        for (uint32_t t = 0; t < nq; ++t)
            if (admitted[t] && !finished[t]) {
                if (active[t] == 0) finished[t] = 1;
                else live++;
            }
        if (next >= nq && live == 0) break;
        if (launches > 100000) { printf("mq no progress\n"); return 1; }
    }
    size_t bad = 0;
    for (uint32_t t = 0; t < nq; ++t)
        for (uint32_t v = 0; v < n; ++v) bad += dist[t][v] != want[(size_t)t * n + v];
    printf("mq delta=%u NB=%d per=%u stagger=%u launches=%u rounds=%u err=%u bad=%zu relaxed=%llu\n", delta, NB, per, stagger,
           launches, ctl.rounds_done, ctl.err, bad, ctl.edges_relaxed);
    return bad != 0;
}
