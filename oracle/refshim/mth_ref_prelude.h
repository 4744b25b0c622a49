/*
 * Forced first include when compiling the reference sources here.  Defining
 * the include guard of src/evpFlags.h makes the compiler skip that file, so
 * the physics flags below are the build's configuration: the shipped set
 * (src/evpFlags.h:4-40) minus DD_CU, whose hard-coded Cu constants
 * (src/init.c:821-825) would override the elastic constants of input.in.
 */
#ifndef MTH_REF_PRELUDE_H
#define MTH_REF_PRELUDE_H
#define EVPFLAGS_H
#define NPHMAX 2
#define NSYSMX 12
#define DD_BASED_FLAG
#define FORWARD_PLUS_BACKWARD
#define NR_MODIFIED
#define DD_GND
#define DD_GND_FIRST_ORDER
#define PF_DRX
#define GB_BULGING_ONLY
#endif
