// Stand-in for the part of the reference's method interface that the FVM_TVD_GPU subclass
// uses, for machines without the reference's source tree: the abstract Method with its
// three entry points (src/methods/method.h:6-11) and, through global.h, log(), EXIT(), hLog
// and Parallel (src/global.h:260-291). The same subclass compiles against the reference's
// own method.h and global.h where that tree exists (oracle/Makefile target dropin).
// Test infrastructure only.
#ifndef DROPIN_IFACE_METHOD_H
#define DROPIN_IFACE_METHOD_H

#include "global.h"

class Method {
public:
    virtual void init(char* xmlFileName) = 0;
    virtual void run() = 0;
    virtual void done() = 0;
    virtual ~Method() {}
};

#endif
