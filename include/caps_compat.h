/*
 * caps_compat.h -- the CAPS reference's C++ interface, served by
 * libcaps_gb300.so on one GPU.  Same names, argument meaning and (C++)
 * linkage as the reference headers, so code written against CAPS links
 * against this library instead of multiply.o / communication.o / memory.o /
 * counters.o / matrix.o / library.o.
 *
 *   multiply            multiply.h:13       (multiply.cpp:9-25)
 *   MatDescriptor       matrix.h:8-16       DESC_SIZE matrix.h:18
 *   numEntriesPerProc   matrix.h:47         (matrix.cpp:9-12)
 *   verifyDescriptor    matrix.h:46         (matrix.cpp:3-7)
 *   allocate, deallocate, enoughMemory, setAvailableMemory, getMaxUsedMemory
 *                       memory.h:10-14      (memory.cpp)
 *   initCommunication, initCommunicationAlt, getRank, getComm,
 *   getLog7nProcs, getPFactor, distributeFrom1Proc, collectTo1Proc
 *                       communication.h:10-17,34-35
 *   initTimers, startTimer, stopTimer, printCounters, increase*
 *                       counters.h:5-21
 *   read_timer          library.h:8          SEVEN library.h:5
 *   mult                cholesky/mult.h:6   (cholesky/mult.cpp:11-28, one rank)
 *   rectMM              rect-class/rectmm.h:1 (rect-class/rectmm.cpp:24-72, one rank)
 *
 * Differences, all forced by one GPU per process:
 *   - one rank: getRank() = 0, getLog7nProcs() = 0, getPFactor() = 1;
 *   - allocate() returns page-locked host memory so multiply() stages its
 *     copies at full PCIe/C2C speed (falls back to malloc);
 *   - multiply() copies A, B to the GPU, runs the Strassen recursion there
 *     and copies C back; the form (FP64 or split) is chosen with
 *     caps_compat_set_form();
 *   - a bad pattern prints "Invalid pattern" and exits(-1) as the reference
 *     does (multiply.cpp:100-104).
 */
#ifndef CAPS_COMPAT_H
#define CAPS_COMPAT_H

struct MatDescriptor {
    int lda;
    int nrec;
    int nproc;
    int nprocr;
    int nprocc;
    int nproc_summa;
    int bs;
};

const int DESC_SIZE = 7;
const int SEVEN = 7;

void multiply(double *A, double *B, double *C, MatDescriptor desc, char *pattern = 0);

/* The Cholesky subproject's multiply (cholesky/mult.h:6): C = alpha C - A B^T
 * on n x n host arrays in its recursive layout, one rank (x = 1). */
void mult(double *C, double *A, double *B, int n, int x, int r, double alpha = 1.);

/* The rectangular subproject's multiply (rect-class/rectmm.h:1): C = A B on
 * host arrays in its block layout, one rank (P = 1), DFS steps; see
 * caps_rect_mm_host. */
void rectMM(double *A, double *B, double *C, int m, int n, int k, int P, int r, char *patt, int *divPatt);

void verifyDescriptor(MatDescriptor desc);
long long numEntriesPerProc(MatDescriptor desc);

double *allocate(long long s);
void deallocate(double *A, long long s);
bool enoughMemory(long long memNeeded);
void setAvailableMemory(long long am);
double getMaxUsedMemory();

void initCommunication(int *argc, char ***argv, int randomize = 0);
void initCommunicationAlt(int *argc, char ***argv, int randomize = 0);
int getRank();
/* communication.h:12 declares `MPI_Comm getComm()`.  On one rank the value is
 * MPI_COMM_WORLD of the one-rank MPI stand-in the drivers compile against,
 * where MPI_Comm is an int (0).  A return type is not part of a C++ symbol
 * name, so callers built against the reference header link to this one; a
 * caller whose mpi.h makes MPI_Comm a pointer type must not use the value. */
int getComm();
int getLog7nProcs();
int getPFactor();
void distributeFrom1Proc(MatDescriptor desc, double *O, double *I);
void collectTo1Proc(MatDescriptor desc, double *O, double *I);

void increaseAdditions(long long n);
void increaseMultiplications(long long n);
void increaseMessages(long long n);
void increaseWords(long long n);
void setExecutionType(int nrec, const char *type);
void initTimers();
void startTimer(int type);
void stopTimer(int type);
const int TIMER_COMM = 0;
const int TIMER_ADD = 1;
const int TIMER_MUL = 2;
const int TIMER_REARRANGE = 3;
const int TIMER_COMM_SUMMA = 4;
const int NUM_TIMERS = 5;
void printCounters(double t, MatDescriptor desc);
void printCounters(MatDescriptor desc);

double read_timer();

/* GB300 additions (no reference counterpart). */
extern "C" {
/* form: 0 = FP64 (plain), 1 = split; slices 0 = automatic */
void caps_compat_set_form(int form, int slices);
/* returns the status of the last multiply() (caps_status) */
int caps_compat_last_status(void);
}

#endif
