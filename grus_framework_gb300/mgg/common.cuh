// common.cuh -- drop-in for the reference's include/common.cuh: the types,
// constants and macros the Grus samples use (vtx_t, weight_t, INFINIT,
// BLOCK_SIZE, ALPHA, EPSILON, TID_1D, H_ERR, the frontier/graph enums and the
// std names re-exported through namespace mgg), with the same values.
#ifndef GRUS_MGG_COMMON_CUH
#define GRUS_MGG_COMMON_CUH

#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <cstring>
#include <fstream>
#include <iostream>
#include <limits>
#include <sstream>
#include <string>
#include <vector>

namespace mgg {
namespace {

#define BLOCK_SIZE 512
#define ALPHA 0.85
#define EPSILON 0.01

using std::cout;
using std::endl;
using std::flush;
using std::ifstream;
using std::ofstream;
using std::string;
using std::stringstream;
using std::to_string;
using std::vector;

using uint = unsigned int;
using vtx_t = unsigned int;     // vertex ids and CSR offsets are 32-bit
using weight_t = unsigned int;
using ulong = unsigned long;

const unsigned int INFINIT = std::numeric_limits<uint>::max() - 1;

#define TID_1D (threadIdx.x + blockIdx.x * blockDim.x)
#define TOTAL_THREADS_1D (gridDim.x * blockDim.x)

// The samples' error check: report and end the program, as the reference's
// H_ERR does.  (The C ABI underneath never exits; it returns status codes.)
inline void HandleError(cudaError_t err, const char *file, int line) {
  if (err != cudaSuccess) {
    printf("%s in %s at line %d\n", cudaGetErrorString(err), file, line);
    fflush(stdout);
    exit(EXIT_FAILURE);
  }
}
#define H_ERR(err) (HandleError(err, __FILE__, __LINE__))

enum Memtype { normal, um };
enum graphFmt { CSR, CSC };
enum subgraphFmt { NORMAL, COMPRESSED };
enum frontierType { BDF_AUTO, BDF, WL, BITMAP };

}  // namespace
}  // namespace mgg

#endif
