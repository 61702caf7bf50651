/*
 * ORACLE — test infrastructure, not product code.
 *
 * A command-line driver around the reference DMR program's OWN host code,
 * compiled from the reference sources where they lie (oracle/Makefile's
 * `ref_dmr` target passes the reference directory with -I; nothing of the
 * reference is copied here).  With the configuration dmr.cu:34-43 sets
 * before its includes, it runs the reference's
 *   readNodes / readTriangles   (helpers.h:5-63: <base>.node, .ele, .poly)
 * and dumps what they parsed (node x/y as float32, triangle rows as uint32,
 * perimeter segments included with INVALIDID as third node) next to
 * <out-prefix>, then fills the reference's result record (myresult.h:22-34)
 * from the arguments and calls its getname / writeResult (myresult.h:13-52),
 * which append the row to result.vi in the working directory.  No GPU code
 * is called.
 *
 * usage: ref_dmr_io <path/base> <out-prefix> <path/exename> <i_ntri> <i_bad>
 *                   <o_ntri> <o_bad> <iterations> <runtime> <time>
 */
#include "common.h"

#define MINANGLE 25
#define PI 3.14159265358979323846
#define FORD float
#define DIMSTYPE unsigned
#define INVALIDID 1234567890
#define MAXID INVALIDID
#include "helpers.h"
#include "myresult.h"

static void dump(const std::string &path, const void *a, size_t bytes) {
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) { perror(path.c_str()); exit(2); }
    if (bytes && fwrite(a, 1, bytes, f) != bytes) { perror(path.c_str()); exit(2); }
    fclose(f);
}

int main(int argc, char **argv) {
    if (argc != 11) {
        fprintf(stderr, "usage: %s <path/base> <out> <path/exe> <i_ntri> <i_bad> <o_ntri> <o_bad> <it> <runtime> <time>\n",
                argv[0]);
        return 1;
    }
    FORD *nodex = nullptr, *nodey = nullptr;
    unsigned nnodes = 0, ntriangles = 0, *tnodes = nullptr;
    readNodes(argv[1], nodex, nodey, nnodes);
    readTriangles(argv[1], tnodes, ntriangles, nnodes);
    const std::string out = argv[2];
    dump(out + ".x", nodex, (size_t)nnodes * sizeof(FORD));
    dump(out + ".y", nodey, (size_t)nnodes * sizeof(FORD));
    dump(out + ".tri", tnodes, (size_t)ntriangles * 3 * sizeof(unsigned));
    FILE *m = fopen((out + ".meta").c_str(), "w");
    fprintf(m, "nnodes=%u\nntriangles=%u\n", nnodes, ntriangles);
    fclose(m);
    getname(myresult.fname, argv[3]);
    getname(myresult.ipname, argv[1]);
    myresult.i_ntriangles = (unsigned)strtoul(argv[4], nullptr, 10);
    myresult.i_bad = (unsigned)strtoul(argv[5], nullptr, 10);
    myresult.o_ntriangles = (unsigned)strtoul(argv[6], nullptr, 10);
    myresult.o_bad = (unsigned)strtoul(argv[7], nullptr, 10);
    myresult.iteration = (unsigned)strtoul(argv[8], nullptr, 10);
    myresult.runtime = strtof(argv[9], nullptr);
    myresult.time = strtof(argv[10], nullptr);
    writeResult();
    return 0;
}
