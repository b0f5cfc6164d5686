/*
 * lapacke.h -- the header name zml's src/c.zig:3 includes (@cInclude
 * "lapacke.h") when built with -Dlink_lapacke; it resolves to this
 * library's LAPACKE-shaped declarations.
 */
#ifndef ZML_GB300_LAPACKE_H
#define ZML_GB300_LAPACKE_H
#include "clapack.h"
#endif
