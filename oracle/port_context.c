/* The srp context of the oracle's shared build (oracle/_build/libsrp_port.so).
 * srp programs define `SRPContext srpContext;` themselves
 * (include/srp/context.h); a ctypes caller cannot, so the shared build of
 * this test-only library provides it. */
#include "srp/context.h"

SRPContext srpContext;
