// Link stubs for building the reference DynELA numerical core without its .dyn interpreter.
//
// Test infrastructure only.  The interpreter (bison/flex) defines `parsedFileName` and
// `isHeritedFrom`; four LAPACK drivers (dpotrf, dpbstf, dtrsen, dtrsna) are referenced by unused
// generalized-eigenvalue routines of the f2c LAPACK but are not shipped with it; xargc/xargv
// belong to libF77's main.c, which is not linked.  None of them is reached by the explicit step.

#include <String.h>
#include <cstdio>
#include <cstdlib>

String parsedFileName = "dnlref.dyn";

unsigned char isHeritedFrom(long, long)
{
  return 0;
}

extern "C" {
int xargc = 0;
char **xargv = 0;

static int missing(const char *name)
{
  fprintf(stderr, "ref_stubs: LAPACK routine %s is not available in this build\n", name);
  abort();
  return -1;
}
int dpotrf_(void) { return missing("dpotrf"); }
int dpbstf_(void) { return missing("dpbstf"); }
int dtrsen_(void) { return missing("dtrsen"); }
int dtrsna_(void) { return missing("dtrsna"); }
}
