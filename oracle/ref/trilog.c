/* Records every call the reference makes to Triangle's triangulate() that
 * meshes a local air loop (no hole points: Scaffold's constructor on a
 * local stencil, src/Scaffold.cpp:150-170), so that the fixtures can hold
 * Triangle's own output for those loops.  TEST INFRASTRUCTURE ONLY: linked
 * into oracle/_ref/ref_driver_trilog with -Wl,--wrap=triangulate; the call
 * itself is passed through unchanged.
 *
 * Record layout (little-endian int32 / float64), appended to $TRI_LOG:
 *   int nIn, int nSeg, int nOut, int nTri,
 *   double in[nIn][2], int seg[nSeg][2], double out[nOut][2], int tri[nTri][3]
 */
#include <stdio.h>
#include <stdlib.h>
#define REAL double
#define VOID int
#define ANSI_DECLARATORS
#include "triangle.h"

void __real_triangulate(char*, struct triangulateio*, struct triangulateio*, struct triangulateio*);

static FILE* logFile = 0;

void __wrap_triangulate(char* sw, struct triangulateio* in, struct triangulateio* out, struct triangulateio* vor)
{
    __real_triangulate(sw, in, out, vor);
    if (in->numberofholes != 0) return;   /* the whole-mesh air mesh */
    if (!logFile) {
        const char* p = getenv("TRI_LOG");
        logFile = fopen(p ? p : "trilog.bin", "wb");
        if (!logFile) return;
    }
    int head[4] = {in->numberofpoints, in->numberofsegments, out->numberofpoints, out->numberoftriangles};
    fwrite(head, sizeof(int), 4, logFile);
    fwrite(in->pointlist, sizeof(double), 2 * (size_t)head[0], logFile);
    fwrite(in->segmentlist, sizeof(int), 2 * (size_t)head[1], logFile);
    fwrite(out->pointlist, sizeof(double), 2 * (size_t)head[2], logFile);
    fwrite(out->trianglelist, sizeof(int), 3 * (size_t)head[3], logFile);
    fflush(logFile);
}
