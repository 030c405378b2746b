// The packed-operator solve for R = 4 and 8 right-hand sides: solve.cu compiled a
// second time with GB_SOLVE_MULTI_RHS defined, which instantiates only those R and
// exports gb::solve_entry_multi / apply_entry_multi / set_wait_limit_multi to the
// main unit (the C entry points live there).  Two units, built in parallel.
#define GB_SOLVE_MULTI_RHS 1
#include "solve.cu"
