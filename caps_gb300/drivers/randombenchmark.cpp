// randombenchmark for one GB300: same flags and report as the CAPS driver
// (randombenchmark.cpp:24-100): -s size (required), -b block size (1),
// -r recursive steps (default floor(log2(s/512))), -m MB / -k KB available,
// -p pattern, --random seed.  Inputs are 2*drand48()-1 in layout order, A
// then B.  GB300 additions: --form plain|split, --slices n, --reps n
// (repeat the timed multiply, report the best).
#include "../../include/caps_compat.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>

static int find_option(int argc, char **argv, const char *option) {
    for (int i = 1; i < argc; i++)
        if (strcmp(argv[i], option) == 0) return i;
    return -1;
}
static int read_int(int argc, char **argv, const char *option, int default_value) {
    int i = find_option(argc, argv, option);
    if (i >= 0 && i < argc - 1) return atoi(argv[i + 1]);
    return default_value;
}
static char *read_string(int argc, char **argv, const char *option, char *default_value) {
    int i = find_option(argc, argv, option);
    if (i >= 0 && i < argc - 1) return argv[i + 1];
    return default_value;
}

static const int MIN_STRASSEN = 512;

int main(int argc, char **argv) {
    int randomize = read_int(argc, argv, "--random", 0);
    initCommunicationAlt(&argc, &argv, randomize);
    initTimers();
    int size = read_int(argc, argv, "-s", -1);
    if (size == -1) {
        printf("Must specify the matrix size desired with -s\n");
        exit(-1);
    }
    int bsReq = read_int(argc, argv, "-b", 1);
    int nrecReq = read_int(argc, argv, "-r", -1);
    char *pattern = read_string(argc, argv, "-p", NULL);
    // -m MB or -k KB; kept in 64 bits (the reference's int overflows past 16 GB)
    long long mem_kb = (long long)read_int(argc, argv, "-m", 1536) * 1024;
    if (find_option(argc, argv, "-k") >= 0) mem_kb = read_int(argc, argv, "-k", 0);
    setAvailableMemory(mem_kb * 128);  // KB -> doubles
    char *form = read_string(argc, argv, "--form", (char *)"plain");
    int slices = read_int(argc, argv, "--slices", 0);
    int reps = read_int(argc, argv, "--reps", 1);
    caps_compat_set_form(strcmp(form, "split") == 0 ? 1 : 0, slices);

    if (nrecReq == -1) {
        int rsize = size / MIN_STRASSEN;
        nrecReq = 0;
        while (rsize > 1) {
            nrecReq += 1;
            rsize /= 2;
        }
        printf("Setting nrec=%d\n", nrecReq);
    }
    printf("Benchmarking size %d\n", size);
    MatDescriptor desc;
    desc.lda = size;
    desc.nrec = nrecReq;
    desc.bs = bsReq;
    desc.nprocr = 1;
    desc.nprocc = 1;
    desc.nproc = 1;
    desc.nproc_summa = getPFactor();

    long long ne = numEntriesPerProc(desc);
    double *A = allocate(ne), *B = allocate(ne), *C = allocate(ne);
    for (long long i = 0; i < ne; i++) A[i] = 2 * drand48() - 1;
    for (long long i = 0; i < ne; i++) B[i] = 2 * drand48() - 1;

    double best = 1e300;
    for (int r = 0; r < reps; r++) {
        if (r > 0) initTimers();
        double t0 = read_timer();
        multiply(A, B, C, desc, pattern);
        double t1 = read_timer();
        if (t1 - t0 < best) best = t1 - t0;
    }
    deallocate(A, ne);
    deallocate(B, ne);
    printCounters(best, desc);
    deallocate(C, ne);
    return 0;
}
