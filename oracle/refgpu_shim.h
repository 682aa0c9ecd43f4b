// Test infrastructure only: CUDA 13 takes a cudaMemLocation and flags in cudaMemPrefetchAsync;
// the reference host code (built only to extract its device code) uses the older 3-argument form.
#include <cuda_runtime.h>
#define cudaMemPrefetchAsync(p, s, d) cudaMemPrefetchAsync((p), (s), cudaMemLocation{cudaMemLocationTypeDevice, (d)}, 0)
