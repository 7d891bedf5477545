// No-op definitions of the reference's CUDA shim entry points
// (cudaCode/*.cuh).  The harness runs the CPU path (-gpu_start=0), where the
// worker still calls the initialisers and the precompute launchers; on a
// machine without a visible GPU their effect is nil, which these stand-ins
// reproduce without compiling or running any reference device code.
namespace tjn {
void init(float*, float*, float*, float*, unsigned int*, unsigned int*, unsigned int*, unsigned int*,
          unsigned int*, unsigned int*, unsigned int*, unsigned int*, unsigned int, unsigned int,
          unsigned int*, unsigned int*, unsigned int*, unsigned int*, char*, float*, unsigned int*,
          unsigned int*) {}
float deltaSum(unsigned int, unsigned int) { return 0.f; }
void g_function_compr(unsigned int, unsigned int) {}
void g_function_pr(unsigned int, unsigned int) {}
void OutMirrorSyncToMaster(unsigned int) {}
void value2last(float*, float*, unsigned int*, int) {}
}  // namespace tjn
namespace tjnpr_precompute {
void init_subgraph(float*, float*, unsigned int*, unsigned int*, unsigned int*, unsigned int*,
                   unsigned int, bool*) {}
int compute(unsigned int, double) { return 1; }
}  // namespace tjnpr_precompute
namespace tjnpr_seg {
void init(float*, float*, float*, float*, unsigned int*, unsigned int*, unsigned int*, unsigned int*,
          unsigned int*, unsigned int*, unsigned int*, unsigned int*, unsigned int, unsigned int,
          unsigned int, unsigned int, unsigned int, unsigned int*, unsigned int*, unsigned int*,
          unsigned int*, char*, float*, unsigned int*, unsigned int*, unsigned int*, unsigned int*,
          unsigned int*, unsigned int*) {}
void g_function_pr(unsigned int) {}
float deltaSum(unsigned int, unsigned int) { return 0.f; }
void g_function_compr(unsigned int, unsigned int*, float*) {}
void OutMirrorSyncToMaster(unsigned int) {}
}  // namespace tjnpr_seg
namespace tjnsssp {
void init(unsigned int*, int*, unsigned int*, int*, int*, unsigned int*, int, unsigned int*,
          unsigned int*, unsigned int*, unsigned int, unsigned int*, int*, unsigned int*,
          unsigned int*, unsigned int*, int*, unsigned int*, unsigned int*, unsigned int*,
          unsigned int*, char*) {}
void g_function(unsigned int*, unsigned int) {}
void g_function_compr(unsigned int*, unsigned int) {}
}  // namespace tjnsssp
namespace tjnsssp_precompute {
void init_subgraph(unsigned int*, unsigned int*, int*, unsigned int*, unsigned int) {}
void init_modified(unsigned int*, int*, unsigned int*, int*, unsigned int*) {}
void compute(unsigned int) {}
}  // namespace tjnsssp_precompute
