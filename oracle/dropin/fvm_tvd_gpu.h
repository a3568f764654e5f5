// The Method subclass a maintainer adds to cfd-2d (as src/methods/fvm_tvd_gpu.h) so that
// the reference's own Solver runs FVM_TVD, FVM_TVD_IMPLICIT and FEM_RKDG tasks on the GPU
// through libcfd2d_gpu.so. It derives from the reference's Method (src/methods/method.h:6-11)
// and compiles against the reference's method.h and global.h; the library is reached only
// through its C ABI (include/cfd2d.h).
//
//   init(xml)  -> cfd2d_create   (FVM_TVD::init: task.xml, mesh files, initial state)
//   run()      -> cfd2d_run      (FVM_TVD::run: the step loop, res_%010d.vtk files, log lines)
//   done()     -> cfd2d_destroy  (FVM_TVD::done)
//
// A failed call is reported the reference's way: the message through log() and EXIT(1)
// (src/global.cpp:32-55). The reference's log() hands its argument list to vprintf and
// vfprintf both, so it is given a complete line with no conversions in it.
#ifndef FVM_TVD_GPU_H
#define FVM_TVD_GPU_H

#include <stdio.h>

#include "cfd2d.h"
#include "method.h"

class FVM_TVD_GPU : public Method {
public:
    virtual void init(char* xmlFileName) {
        if (cfd2d_create(xmlFileName, &h) != CFD2D_OK) fail();
    }
    virtual void run() {
        // VTK every FILE_OUTPUT_STEP, a log line every LOG_OUTPUT_STEP; the two warnings
        // leave a state the caller may still want
        const int rc = cfd2d_run(h);
        if (rc != CFD2D_OK && rc != CFD2D_ERR_NEWTON_CAP && rc != CFD2D_ERR_NONPHYSICAL) fail();
    }
    virtual void done() {
        cfd2d_destroy(h);
        h = 0;
    }

private:
    cfd2d_t* h = 0;
    void fail() {
        char msg[512], line[600];
        cfd2d_last_error(msg, sizeof msg);
        snprintf(line, sizeof line, "ERROR: %s\n", msg);
        for (char* c = line; *c; c++)
            if (*c == '%') *c = ' ';
        log(line);
        EXIT(1);
    }
};

#endif
