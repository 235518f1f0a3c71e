// print.cuh -- drop-in for the reference's include/print.cuh: the LOG macro
// (file:line prefix, host and device), PrintResults, SaveResults (one
// "<index> <value>" line per vertex, iostream default formatting) and topRank.
#ifndef GRUS_MGG_PRINT_CUH
#define GRUS_MGG_PRINT_CUH

#include <algorithm>

#include "common.cuh"

#define LOG(...) print::myprintf(__FILE__, __LINE__, __VA_ARGS__)
#define VNAME(value) (#value)

namespace mgg {
namespace print {

template <typename... Args>
__host__ __device__ __forceinline__ void myprintf(const char *file, int line, const char *fmt,
                                                  Args... args) {
#if defined(__CUDA_ARCH__)
  if (TID_1D != 0) return;
  printf("%s:%d GPU: ", file, line);
#else
  printf("%s:%d HOST: ", file, line);
#endif
  if constexpr (sizeof...(Args) == 0) printf("%s", fmt);
  else printf(fmt, args...);
}

template <typename T>
void PrintResults(T *results, uint n) {
  cout << "First " << n << " elements of results :\n[";
  for (uint i = 0; i < n; i++) cout << (i ? " " : "") << i << ":" << results[i];
  cout << "]\n";
}

// `results` must be host-readable (the samples pass managed arrays).
template <typename T>
void SaveResults(string filepath, T *results, uint n) {
  cout << "Saving the results into the following file:\n>> " << filepath << endl;
  ofstream outfile(filepath);
  for (uint i = 0; i < n; i++) outfile << i << " " << results[i] << "\n";
  outfile.close();
  cout << "Done saving.\n";
}

template <typename VertexId, typename Value>
struct RankPair {
  VertexId vertex_id;
  Value page_rank;
  RankPair(VertexId v, Value r) : vertex_id(v), page_rank(r) {}
};

template <typename P>
bool PRCompare(P a, P b) {
  return a.page_rank > b.page_rank;
}

inline void topRank(float *results, uint n, uint m) {
  std::vector<RankPair<uint, float>> v;
  v.reserve(n);
  for (uint i = 0; i < n; ++i) v.emplace_back(i, results[i]);
  std::stable_sort(v.begin(), v.end(), PRCompare<RankPair<uint, float>>);
  for (uint i = 0; i < m && i < n; ++i)
    printf("Vertex ID: %lld, PageRank: %.8le\n", (long long)v[i].vertex_id, (double)v[i].page_rank);
}

}  // namespace print
}  // namespace mgg
#endif
