/* The public header compiles as C (a C caller's view of the ABI). */
#include "csimgpu.h"

int main(void) {
  const char* v = csg_version();
  return v ? 0 : 1;
}
