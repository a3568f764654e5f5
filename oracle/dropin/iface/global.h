// Stand-in declarations of the reference's log(), EXIT(), hLog and Parallel
// (src/global.h:260-291) with the same names and signatures; see method.h beside it.
#ifndef DROPIN_IFACE_GLOBAL_H
#define DROPIN_IFACE_GLOBAL_H

#include <stdio.h>

extern FILE* hLog;
void log(char* format, ...);
void EXIT(int err);

struct Parallel {
    static int procCount, procId;
    static void init(int* argc, char*** argv);
    static void done();
};

#endif
