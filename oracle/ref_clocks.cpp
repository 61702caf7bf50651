/*
 * ORACLE — test infrastructure, not product code.
 *
 * Runs the reference's own load-balance estimate, combineClocks
 * (metrics.h:68-84, with getminIndex / getmaxIndex, metrics.h:1-24),
 * compiled from the reference sources where they lie (the Makefile passes
 * the reference directory with -I; nothing of the reference is copied here).
 *
 * stdin: a count followed by that many per-block clock values.
 * stdout: the estimate, then the SM index of every block.
 */
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
using namespace std;
#include "metrics.h"

int main() {
    unsigned len = 0;
    if (scanf("%u", &len) != 1) return 1;
    unsigned *ary = (unsigned *)malloc((len ? len : 1) * sizeof(unsigned));
    for (unsigned i = 0; i < len; ++i)
        if (scanf("%u", &ary[i]) != 1) return 1;
    unsigned *aindex = nullptr;
    char pad[] = "clocks";
    const unsigned long est = combineClocks(ary, len, aindex, pad);
    printf("%lu\n", est);
    for (unsigned i = 0; i < len; ++i) printf("%u%c", aindex[i], i + 1 < len ? ' ' : '\n');
    return 0;
}
