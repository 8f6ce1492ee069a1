/* Compiles the public header as plain C99 and calls the library through it without a GPU:
 * version and status strings, and argument validation that runs before any CUDA call. */
#include <stdio.h>
#include <string.h>

#include "addft_gb300.h"

static int fail(const char *what) {
  fprintf(stderr, "abi_check: %s (last error: %s)\n", what, addft_last_error());
  return 1;
}

int main(void) {
  if (addft_version() < 1) return fail("version");
  if (strcmp(addft_status_string(ADDFT_OK), "ok") != 0) return fail("status string");
  addft_plan plan = NULL;
  const int32_t miller[6] = {0, 0, 0, 9, 0, 0}; /* two G on the same point of a 9^3 box */
  if (addft_plan_create(&plan, 9, 9, 9, 2, miller) != ADDFT_INVALID_ARG) return fail("aliased sphere accepted");
  if (addft_plan_create(&plan, 7, 9, 9, 2, miller) != ADDFT_UNSUPPORTED) return fail("non-smooth box accepted");
  if (addft_hpsi(NULL, ADDFT_F32, 1, 4, NULL, NULL, NULL, 0, NULL, NULL, NULL, NULL, 0, NULL) != ADDFT_INVALID_ARG)
    return fail("hpsi without a plan accepted");
  if (addft_ffi_eigh_lowest(1, 4, 5, NULL, NULL, NULL, NULL, 0, NULL) != ADDFT_INVALID_ARG)
    return fail("nband > n accepted");
  if (addft_ffi_scatter(ADDFT_F64, -1, 4, 8, NULL, NULL, NULL, NULL) != ADDFT_INVALID_ARG)
    return fail("negative batch accepted");
  if (addft_hpsi_noalloc_max_scratch_bytes() == 0) return fail("no-allocation scratch size");
  printf("abi_check ok: version %d\n", addft_version());
  return 0;
}
