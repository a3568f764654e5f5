// Test harness: the reference's main (src/main.cpp:10-39) with the method factory of
// Solver::initMethod (src/methods/solver.cpp:13-61) as a maintainer extends it for the GPU
// (the FVM_TVD_GPU registration lines of the integration notes), linked with
// libcfd2d_gpu.so. Built two ways (oracle/Makefile): against the reference's own
// method.h / global.h with its global and grid objects (target dropin, where the
// reference's source tree exists), and against the stand-ins in iface/ (target
// dropin-standin, anywhere). Every method name the library runs maps to FVM_TVD_GPU;
// any other is the reference's "unknown method" error (exit -1).
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fvm_tvd_gpu.h"
#include "global.h"

// The method attribute of <task ...> in the task file (Solver::initMethod reads it with
// TinyXML; the harness needs only this one attribute).
static bool task_method(const char* fileName, char* name, size_t n) {
    FILE* f = fopen(fileName, "rb");
    if (!f) return false;
    char buf[4096];
    const size_t len = fread(buf, 1, sizeof buf - 1, f);
    fclose(f);
    buf[len] = 0;
    const char* t = strstr(buf, "<task");
    const char* m = t ? strstr(t, "method") : 0;
    const char* q = m ? strpbrk(m, "\"'") : 0;
    if (!q) return false;
    const char* e = strchr(q + 1, *q);
    if (!e || (size_t)(e - q - 1) >= n) return false;
    memcpy(name, q + 1, e - q - 1);
    name[e - q - 1] = 0;
    return true;
}

static Method* initMethod(char* fileName) {
    char methodName[64];
    if (!task_method(fileName, methodName, sizeof methodName)) {
        char line[] = "ERROR: cannot read the task file\n";
        log(line);
        exit(1);
    }
    Method* m = 0;
    if (strcmp("FVM_TVD_GPU", methodName) == 0 || strcmp("FVM_TVD", methodName) == 0 ||
        strcmp("FVM_TVD_IMPLICIT", methodName) == 0 || strcmp("FEM_RKDG", methodName) == 0) {
        m = new FVM_TVD_GPU();
    } else {
        char line[] = "ERROR: unknown method.\n";
        log(line);
        exit(-1);
    }
    m->init(fileName);
    return m;
}

int main(int argc, char** argv) {
    Parallel::init(&argc, &argv);
    hLog = fopen("task.log", "w");
    char task[] = "task.xml";
    Method* method = initMethod(task);
    method->run();   // Solver::runMethod
    method->done();  // Solver::destroyMethod
    delete method;
    fclose(hLog);
    Parallel::done();
    return 0;
}
