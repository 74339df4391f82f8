/* The C ABI header as a C caller (a cgo, JNI or ctypes binding) sees it:
 * it compiles as strict C99 and links against libphase_gb300 with no C++
 * runtime in the caller. */
#include <stdio.h>

#include "phase_gb300.h"

int main(void) {
  pg_solver_cfg c;
  pg_solver_default_cfg(&c);
  printf("tolerance %g max_iters %d\n", c.tolerance, c.max_iters);
  return c.max_iters == 500 ? 0 : 1;
}
