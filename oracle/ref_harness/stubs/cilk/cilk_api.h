#ifndef SG_REF_CILK_API_STUB_H_
#define SG_REF_CILK_API_STUB_H_
#include <omp.h>
inline int __cilkrts_get_worker_number() { return omp_get_thread_num(); }
inline int __cilkrts_get_nworkers() { return omp_get_max_threads(); }
inline int __cilkrts_set_param(const char*, const char*) { return 0; }
#endif
