/* Runs the mesh refinement kernels' text (dmr.cu) round by round on a mesh
 * in dir/{x,y}.bin (float64) and dir/{tri,nbr}.bin (uint32), the way
 * gga_mesh_refine launches them, and writes the refined arrays and the stop
 * word to dir/out_*.bin; once few triangles are bad, the one-block tail
 * kernel runs the rounds, handing back when the worklist outgrows tail_max.
 * args: dir G BS PBS batch_cap tcap cos_bound(hex) [tail_max [pf_max]] */
#include "kernel_dmr.inc"
static std::vector<double> rdd(const std::string &p) {
    std::ifstream f(p, std::ios::binary); f.seekg(0, std::ios::end); size_t n = f.tellg() / 8; f.seekg(0);
    std::vector<double> v(n); f.read((char *)v.data(), n * 8); return v;
}
template <class T> static void wr(const std::string &p, const T *v, size_t n) {
    std::ofstream f(p, std::ios::binary); f.write((const char *)v, n * sizeof(T));
}
#define LAUNCH_PF(PF, NB, BS) run_grid(NB, BS, [&](int b) { switch (b) { case 0: k_plan<PF, 0>(a); break; default: k_plan<PF, 1>(a); } })
#define LAUNCH(K, NB, BS) run_grid(NB, BS, [&](int b) { switch (b) { case 0: K<0>(a); break; case 1: K<1>(a); break; case 2: K<2>(a); break; default: K<3>(a); } })
int main(int argc, char **argv) {
    if (argc < 8) return 1;
    const std::string d = argv[1];
    const int G = atoi(argv[2]), BS = atoi(argv[3]), PBS = atoi(argv[4]);
    const uint32_t bcap = (uint32_t)atol(argv[5]), tcap = (uint32_t)atol(argv[6]);
    const double cb = strtod(argv[7], nullptr);
    const long tmax = argc > 8 ? atol(argv[8]) : 2048;
    const long pfmax = argc > 9 ? atol(argv[9]) : 32768;
    auto x0 = rdd(d + "/x.bin"), y0 = rdd(d + "/y.bin");
    auto t0 = rd(d + "/tri.bin"), n0 = rd(d + "/nbr.bin");
    const uint32_t npts = x0.size(), ntri = t0.size() / 3, pcap = npts + (tcap - ntri);
    const uint32_t B = bcap < tcap ? bcap : tcap;
    std::vector<double> x(pcap), y(pcap), px(B), py(B);
    std::vector<float4> pq(pcap);
    std::vector<uint32_t> tri(3 * (size_t)tcap), nbr(3 * (size_t)tcap), bad(tcap), work(B), pm(B), pc((size_t)CAV_MAX * B),
        pw(B), bsum(3 * G), lock(tcap, 0), wlist(B), wtri(B);
    std::vector<uint4> pf((size_t)FAN_MAX * B);
    std::vector<unsigned long long> owner(tcap, 0), ring(tcap, 0);
    std::copy(x0.begin(), x0.end(), x.begin());
    std::copy(y0.begin(), y0.end(), y.begin());
    std::copy(t0.begin(), t0.end(), tri.begin());
    std::copy(n0.begin(), n0.end(), nbr.begin());
    DmrState st;
    memset(&st, 0, sizeof st);
    st.npts = npts; st.ntri = ntri; st.pcap = pcap; st.tcap = tcap; st.bcap = B; st.max_rounds = MAX_ROUNDS;
    DmrArgs a;
    a.x = x.data(); a.y = y.data(); a.tri = tri.data(); a.nbr = nbr.data(); a.bad = bad.data(); a.owner = owner.data(); a.ring = ring.data(); a.lock = lock.data();
    a.wlist = wlist.data(); a.wtri = wtri.data();
    a.work = work.data(); a.p_mode = pm.data(); a.p_px = px.data(); a.p_py = py.data(); a.p_cav = pc.data();
    a.p_fan = pf.data(); a.p_win = pw.data(); a.bsum = bsum.data(); a.st = &st; a.cos_bound = cb; a.B = B; a.G = G;
    a.pq = pq.data(); a.cos_bound_f = (float)cb;
    a.tail_max = (uint32_t)std::min<long>(std::min<long>(tmax, B), TAIL_SORT);
    a.pf_max = (uint32_t)pfmax;
    uint32_t sbits = 0;
    run_grid(G, BS, [&](int b) { switch (b) { case 0: k_shadow<0>(a, &sbits); break; case 1: k_shadow<1>(a, &sbits); break; case 2: k_shadow<2>(a, &sbits); break; default: k_shadow<3>(a, &sbits); } });
    a.S = __uint_as_float(sbits) * (1.0f + 1.0f / 1048576.0f) + 1e-30f;
    LAUNCH(k_mark_all, G, BS);
    uint32_t tails = 0;
    for (uint32_t r = 0; st.stop == STOP_NONE && r < 4096; ++r) {
        LAUNCH(k_bad_count, G, BS);
        LAUNCH(k_bad_gather, G, BS);
        LAUNCH(k_decide, 1, 32);
        LAUNCH_PF(false, 2, PBS);
        LAUNCH_PF(true, 2, PBS);
        LAUNCH(k_resolve0, 2, PBS);
        LAUNCH(k_reclaim, 2, PBS);
        LAUNCH(k_resolve1, G, BS);
        LAUNCH(k_compact, G, BS);
        LAUNCH(k_commit, 2, PBS);
        LAUNCH(k_finish, 1, 1);
        if (st.stop == STOP_NONE && st.tail) {
            LAUNCH(k_tail, 1, BS);
            ++tails;
        }
    }
    wr(d + "/out_x.bin", x.data(), st.npts);
    wr(d + "/out_y.bin", y.data(), st.npts);
    wr(d + "/out_tri.bin", tri.data(), 3 * (size_t)st.ntri);
    wr(d + "/out_nbr.bin", nbr.data(), 3 * (size_t)st.ntri);
    printf("stop %u rounds %u npts %u ntri %u nbad %u bad_in %u ins %llu splits %llu failed %llu err %u tails %u\n",
           st.stop, st.round, st.npts, st.ntri, st.nbad, st.bad_in, st.insertions, st.splits, st.failed, st.err, tails);
    return 0;
}
