// fromfile1 for one GB300: same flags and output as the CAPS known-answer
// driver (fromfile1.cpp:11-164): -i input (n, then the n rows of A and of B),
// -b block size and -r recursive steps (both required), -o output file,
// -c check file ("Maximum deviation %e"), -m MB / -k KB, -p pattern.
// GB300 additions: --form plain|split, --slices n.
#include "../../include/caps_compat.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

// Whole-file text reading: one read, then strtod over the buffer (the
// reference reads element by element with fscanf, fromfile1.cpp:45-57, which
// takes minutes for matrices in the thousands).
struct TextNumbers {
    char *buf = nullptr;
    char *p = nullptr;
    bool open(const char *path) {
        FILE *f = fopen(path, "rb");
        if (!f) return false;
        fseek(f, 0, SEEK_END);
        long sz = ftell(f);
        fseek(f, 0, SEEK_SET);
        buf = (char *)malloc((size_t)sz + 1);
        size_t got = fread(buf, 1, (size_t)sz, f);
        buf[got] = 0;
        fclose(f);
        p = buf;
        return true;
    }
    // next number; false at the end of the text or on a token that is not one
    bool next(double *v) {
        char *e = nullptr;
        *v = strtod(p, &e);
        if (e == p) return false;
        p = e;
        return true;
    }
    ~TextNumbers() { free(buf); }
};

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

int main(int argc, char **argv) {
    int randomize = read_int(argc, argv, "--random", 0);
    initCommunication(&argc, &argv, randomize);
    initTimers();
    MatDescriptor desc;
    long long mem = (long long)read_int(argc, argv, "-m", 1536) * 1024;
    if (find_option(argc, argv, "-k") >= 0) mem = read_int(argc, argv, "-k", 0);
    setAvailableMemory(mem * 128);
    char *inFile = read_string(argc, argv, "-i", NULL);
    char *outFile = read_string(argc, argv, "-o", NULL);
    char *checkFile = read_string(argc, argv, "-c", NULL);
    int bsReq = read_int(argc, argv, "-b", -1);
    int nrecReq = read_int(argc, argv, "-r", -1);
    char *form = read_string(argc, argv, "--form", (char *)"plain");
    caps_compat_set_form(strcmp(form, "split") == 0 ? 1 : 0, read_int(argc, argv, "--slices", 0));
    if (!inFile) {
        printf("Specify input file\n");
        exit(-1);
    }
    TextNumbers in;
    if (!in.open(inFile)) {
        printf("Error opening file: %s\n", inFile);
        exit(-1);
    }
    long long reads = 0;
    double v;
    desc.lda = 0;
    if (in.next(&v)) {
        desc.lda = (int)v;
        reads++;
    }
    long long nn = (long long)desc.lda * desc.lda;
    double *IA = allocate(nn), *IB = allocate(nn);
    for (int M = 0; M < 2; M++) {
        double *X = M == 0 ? IA : IB;
        for (int i = 0; i < desc.lda; i++)
            for (int j = 0; j < desc.lda; j++)
                if (in.next(&v)) {
                    X[i + (long long)j * desc.lda] = v;  // row i of the file is row i of the matrix
                    reads++;
                }
    }
    if (reads != nn * 2 + 1) {
        printf("Error reading file: %s, only read %lld entries\n", inFile, reads);
        exit(-1);
    }
    printf("Read complete\n");
    if (bsReq == -1 || nrecReq == -1) {
        printf("Specify parameters with -b and -r.  Automatic determination of parameters not yet available\n");
        exit(-1);
    }
    desc.nrec = nrecReq;
    desc.bs = bsReq;
    desc.nprocr = desc.nprocc = desc.nproc = 1;
    desc.nproc_summa = getPFactor();
    if (desc.lda % ((1 << desc.nrec) * desc.bs) != 0) {
        printf("Matrix dimension %d is not a multiple of 2^r*bs = %d\n", desc.lda, (1 << desc.nrec) * desc.bs);
        exit(-1);
    }
    long long ne = numEntriesPerProc(desc);
    double *A = allocate(ne), *B = allocate(ne);
    distributeFrom1Proc(desc, A, IA);
    distributeFrom1Proc(desc, B, IB);
    deallocate(IA, nn);
    deallocate(IB, nn);
    double *C = allocate(ne);
    char *pattern = read_string(argc, argv, "-p", NULL);
    double startTime = read_timer();
    multiply(A, B, C, desc, pattern);
    double endTime = read_timer();
    deallocate(A, ne);
    deallocate(B, ne);
    double *OC = allocate(nn);
    collectTo1Proc(desc, OC, C);
    if (checkFile) {
        TextNumbers chk;
        if (!chk.open(checkFile)) {
            printf("Error opening file: %s\n", checkFile);
            exit(-1);
        }
        double CC, error = 0;
        for (int i = 0; i < desc.lda; i++) {
            for (int j = 0; j < desc.lda; j++) {
                if (chk.next(&CC)) {
                    double e = fabs(OC[i + (long long)j * desc.lda] - CC);
                    if (e > error) error = e;
                } else {
                    printf("Error reading verification file\n");
                    exit(-1);
                }
            }
        }
        printf("Maximum deviation %e\n", error);
    } else {
        FILE *oFile = outFile ? fopen(outFile, "w") : stdout;
        for (int i = 0; i < desc.lda; i++) {
            for (int j = 0; j < desc.lda; j++) fprintf(oFile, "%.18le ", OC[i + (long long)j * desc.lda]);
            fprintf(oFile, "\n");
        }
        if (outFile) fclose(oFile);
    }
    printCounters(endTime - startTime, desc);
    deallocate(C, ne);
    deallocate(OC, nn);
    return 0;
}
