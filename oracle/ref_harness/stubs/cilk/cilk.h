// Cilk stand-in: the harness builds the reference with -DOPENMP, so
// parallel_for maps to OpenMP (grape/parallel/parallel.h:81-91).
#ifndef SG_REF_CILK_STUB_H_
#define SG_REF_CILK_STUB_H_
#endif
