// Stand-in definitions for global.h beside it: one process; log() writes the line to
// stdout and to hLog as the reference's does (src/global.cpp:32-46), EXIT() closes the log
// and exits with the code (src/global.cpp:48-53).
#include "global.h"

#include <stdarg.h>
#include <stdlib.h>

FILE* hLog = 0;
int Parallel::procCount = 1;
int Parallel::procId = 0;

void Parallel::init(int*, char***) {}
void Parallel::done() {}

void log(char* format, ...) {
    va_list a, b;
    va_start(a, format);
    va_copy(b, a);
    vprintf(format, a);
    if (hLog) vfprintf(hLog, format, b);
    va_end(b);
    va_end(a);
    fflush(stdout);
    if (hLog) fflush(hLog);
}

void EXIT(int err) {
    if (hLog) fclose(hLog);
    exit(err);
}
