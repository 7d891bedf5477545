// Force-included before every reference translation unit of the harness.
#include <unistd.h>
#include <cilk/cilk.h>
#include <cilk/cilk_api.h>
#include <cilk/reducer_opadd.h>
