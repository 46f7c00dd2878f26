/*
 * ref_globals.c -- definitions of the reference's global variables for the
 * oracle/_ref build of the reference's host C files.  In the reference program
 * these are defined by the main translation unit (cudagaugefix.cu:2, global.h with
 * MAIN_PROGRAM); the host files only declare them.  Test infrastructure only.
 */
#define MAIN_PROGRAM
#include "cudaglobal.h"
#include "global.h"
