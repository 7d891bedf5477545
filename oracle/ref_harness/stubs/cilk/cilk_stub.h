#ifndef SG_REF_CILK_STUB2_H_
#define SG_REF_CILK_STUB2_H_
#endif
