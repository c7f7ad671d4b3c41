// Test infrastructure: prepended to the reference translation unit (code/nans.cpp) when
// the oracle recipe compiles the reference headless (oracle/Makefile, target `ref`).
//
// The reference keeps three solver constants as local literals: restitution Cr = 0.1
// (code/nans.cpp:1154), friction Cf = 0.1f (:1159) and 70 impulse iterations (:1176).
// The recipe rewrites exactly those three initialisers, in a pipe and without writing a
// copy of the source, to read the variables below. Their defaults are the literals, and a
// test checks that the rewritten build equals the unmodified build at the defaults.
#ifndef NANS_REF_HARNESS_PRE_H
#define NANS_REF_HARNESS_PRE_H

#include <cfloat>

static float nans_ref_cr = (float)0.1;
static float nans_ref_cf = 0.1f;
static int nans_ref_iters = 70;

#endif
