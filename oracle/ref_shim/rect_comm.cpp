/*
 * One-rank stand-ins for the rectangular subproject's data exchange
 * (rect-class/communication.h: reduceBy, expandBy), used only to link its
 * unmodified rectmm.cpp and rectsizes.cpp for the oracle build
 * (oracle/build_ref.sh).  Its BFS step, the only caller, needs more than one
 * rank; on one rank the process aborts if it is reached.
 */
#include <cstdio>
#include <cstdlib>

void reduceBy(int, int, double **, double *, int *) {
    std::fprintf(stderr, "rect stand-in: reduceBy needs more than one rank\n");
    std::abort();
}
void expandBy(int, int, double **, double *, int *) {
    std::fprintf(stderr, "rect stand-in: expandBy needs more than one rank\n");
    std::abort();
}
