/* nanos6/debug.h -- the one OmpSs-2 runtime query cpic makes
 * (src/solver.c:304).  TEST INFRASTRUCTURE ONLY. */
#ifndef ORC_SHIM_NANOS6_DEBUG_H
#define ORC_SHIM_NANOS6_DEBUG_H
unsigned int nanos6_get_num_cpus(void);
#endif
