// cfd2d_gpu: the reference's program entry (src/main.cpp:10-39) on the GPU path:
// read task.xml from the working directory, log to task.log and stdout, run the
// task's method (FVM_TVD, FVM_TVD_IMPLICIT or FEM_RKDG) with its file and log
// cadence, free everything. An optional argument names another task file.
#include <cstdio>

#include "cfd2d.h"

int main(int argc, char** argv) {
    const char* task = argc > 1 ? argv[1] : "task.xml";
    char msg[1024];
    cfd2d_set_log_file("task.log");
    cfd2d_t* h = nullptr;
    int rc = cfd2d_create(task, &h);
    if (rc != CFD2D_OK) {
        cfd2d_last_error(msg, sizeof msg);
        std::fprintf(stderr, "ERROR: %s\n", msg);
        return rc;
    }
    rc = cfd2d_run(h);
    if (rc != CFD2D_OK) {
        cfd2d_last_error(msg, sizeof msg);
        std::fprintf(stderr, "WARNING (%d): %s\n", rc, msg);
    }
    cfd2d_destroy(h);
    cfd2d_set_log_file(nullptr);
    return rc == CFD2D_OK ? 0 : rc;
}
