/* The mesh refinement kernels' predicates (dmr.cu: orient_sign,
 * incircle_sign, tri_bad), compiled from their own text, against the plain
 * double expressions the oracle evaluates, on near-degenerate cases: points
 * within relative 1e-3 .. 1e-9 of a circumcircle or of a line, thin and
 * flat triangles, triangles at the resolution of a 50M-triangle unit square
 * and far from the origin.  Prints the number of cases, disagreements (must
 * be 0) and how many cases each filter left to double.  args: cases seed */
#include "kernel_dmr.inc"
#include <random>

static int sgn(double v) { return v > 0 ? 1 : (v < 0 ? -1 : 0); }

int main(int argc, char **argv) {
    const long cases = argc > 1 ? atol(argv[1]) : 100000;
    std::mt19937_64 rng(argc > 2 ? atol(argv[2]) : 1);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    std::vector<double> x(8), y(8);
    std::vector<float4> pq(8);
    std::vector<uint32_t> tri = {0, 1, 2};
    DmrState st;
    memset(&st, 0, sizeof st);
    DmrArgs a;
    memset(&a, 0, sizeof a);
    a.x = x.data(); a.y = y.data(); a.pq = pq.data(); a.tri = tri.data(); a.st = &st;
    long bad_or = 0, bad_ic = 0, bad_an = 0, fb_or = 0, fb_an = 0;
    const double cb = std::cos(25.0 * (3.14159265358979323846 / 180.0));
    a.cos_bound = cb;
    a.cos_bound_f = (float)cb;
    for (long c = 0; c < cases; ++c) {
        /* a frame: origin offset up to `off`, feature size h */
        const int kind = (int)(c % 4);
        const double off = kind == 3 ? 1000.0 : 1.0, h = std::pow(10.0, -1.0 - 3.5 * U(rng));
        const double ox = off * U(rng), oy = off * U(rng);
        /* triangle: random, or thin / flat */
        double tx[3], ty[3];
        for (int i = 0; i < 3; ++i) {
            tx[i] = ox + h * U(rng);
            ty[i] = oy + h * U(rng);
        }
        if (kind == 1) ty[2] = ty[0] + (ty[1] - ty[0]) * (tx[2] - tx[0]) / (tx[1] - tx[0]) + h * 1e-6 * (U(rng) - 0.5);
        double o0 = (tx[1] - tx[0]) * (ty[2] - ty[0]) - (ty[1] - ty[0]) * (tx[2] - tx[0]);
        if (o0 == 0) continue;
        if (o0 < 0) {
            std::swap(tx[1], tx[2]);
            std::swap(ty[1], ty[2]);
        }
        for (int i = 0; i < 3; ++i) {
            x[i] = tx[i];
            y[i] = ty[i];
        }
        /* circumcentre, and a point at relative distance 10^-(3..9) of the circle */
        const double bx = x[1] - x[0], by = y[1] - y[0], cx = x[2] - x[0], cy = y[2] - y[0];
        const double d = 2.0 * (bx * cy - by * cx), b2 = bx * bx + by * by, c2 = cx * cx + cy * cy;
        const double ux = (cy * b2 - by * c2) / d, uy = (bx * c2 - cx * b2) / d;
        const double R = std::sqrt(ux * ux + uy * uy), th = 6.283185307179586 * U(rng);
        const double rel = (U(rng) - 0.5) * std::pow(10.0, -3.0 - 6.0 * U(rng));
        const double px = x[0] + ux + R * (1 + rel) * std::cos(th), py = y[0] + uy + R * (1 + rel) * std::sin(th);
        /* a point near the line through vertices 0 and 1 */
        const double s = U(rng), nrm = std::pow(10.0, -3.0 - 8.0 * U(rng)) * h * (U(rng) - 0.5);
        const double qx = x[0] + s * bx - by * nrm, qy = y[0] + s * by + bx * nrm;
        double S = 0;
        for (int i = 0; i < 3; ++i) S = std::max(S, std::max(std::fabs(x[i]), std::fabs(y[i])));
        a.S = (float)(S * (1.0 + 1.0 / 1048576.0)) + 1e-30f;
        for (int i = 0; i < 3; ++i) pq[i] = fpair_of(x[i], y[i]);
        {
            const float4 pt = fpair_of(px, py);
            const float A = a.S + fmaxf(a.S, fmaxf(fabsf(pt.x), fabsf(pt.y)));
            const double adx = x[0] - px, ady = y[0] - py, bdx = x[1] - px, bdy = y[1] - py, cdx = x[2] - px,
                         cdy = y[2] - py;
            const double ad = adx * adx + ady * ady, bd = bdx * bdx + bdy * bdy, cd = cdx * cdx + cdy * cdy;
            const int want = sgn(adx * (bdy * cd - bd * cdy) - ady * (bdx * cd - bd * cdx) + ad * (bdx * cdy - bdy * cdx));
            bad_ic += incircle_sign(a, 0, 1, 2, px, py, pt, A) != want;
        }
        {
            const float4 qt = fpair_of(qx, qy);
            const float A = a.S + fmaxf(a.S, fmaxf(fabsf(qt.x), fabsf(qt.y)));
            const int want = sgn((x[1] - x[0]) * (qy - y[0]) - (y[1] - y[0]) * (qx - x[0]));
            bad_or += orient_sign(a, 0, 1, pq[0], pq[1], qx, qy, qt, A) != want;
        }
        {
            /* angle test on the triangle: compare with the double rule */
            int want = 0;
            for (int i = 0; i < 3; ++i) {
                const int p = i, q = (i + 1) % 3, r = (i + 2) % 3;
                const double vx = x[q] - x[p], vy = y[q] - y[p], wx = x[r] - x[p], wy = y[r] - y[p];
                if (vx * wx + vy * wy > cb * std::sqrt((vx * vx + vy * vy) * (wx * wx + wy * wy))) want = 1;
            }
            bad_an += (int)tri_bad(a, 0) != want;
            const float A = 2.0f * a.S;
            const float g01x = fdx(pq[1], pq[0]), g01y = fdy(pq[1], pq[0]), g02x = fdx(pq[2], pq[0]),
                        g02y = fdy(pq[2], pq[0]);
            fb_an += angle_small_f(g01x, g01y, g02x, g02y, a.cos_bound_f, A) < 0;
        }
    }
    /* fallback rates of the two geometric filters, measured on the same kinds of cases */
    std::mt19937_64 r2(7);
    for (long c = 0; c < cases / 10; ++c) {
        const double h = std::pow(10.0, -1.0 - 3.5 * U(r2));
        const double ox = U(r2), oy = U(r2);
        for (int i = 0; i < 3; ++i) {
            x[i] = ox + h * U(r2);
            y[i] = oy + h * U(r2);
            pq[i] = fpair_of(x[i], y[i]);
        }
        a.S = 2.0f;
        const double px = ox + h * U(r2), py = oy + h * U(r2);
        const float4 pt = fpair_of(px, py);
        const float A = 4.0f;
        const float u1 = fdx(pq[1], pq[0]), v1 = fdy(pt, pq[0]), u2 = fdy(pq[1], pq[0]), v2 = fdx(pt, pq[0]);
        const float a1 = u1 * v1, a2 = u2 * v2, F = a1 - a2, L = fmax4(u1, v1, u2, v2), D = err_d(L, A);
        fb_or += !(fabsf(F) > 2.01f * (4.0f * D * (L + D) + 3.0f * EPSF * (fabsf(a1) + fabsf(a2))));
    }
    printf("cases %ld orient_wrong %ld incircle_wrong %ld angle_wrong %ld angle_fallback %ld orient_fallback_random %ld\n",
           cases, bad_or, bad_ic, bad_an, fb_an, fb_or);
    return bad_or || bad_ic || bad_an ? 1 : 0;
}
