// Test driver for Program::scatter on the GPU (include/gpugas.h): a user
// program whose scatter writes its edge data, which the next gather reads.
//
//   scatter_driver <in.bin> <out.bin>
// in.bin : int32 nV, nE, then src[nE], dst[nE], uses[nE]
// out.bin: int32 label[nV], uses[nE] (edge-list order, after getResults),
//          iterations
#include <climits>
#include <cstdio>
#include <vector>

#include "gpugas.h"

// Labels start at 3 v and shrink to min(label[src] + uses[edge]) over in-edges; every
// scatter ages the edge by 1 + parity(label[src] + label[dst]).
struct TAging {
  typedef int VertexData;
  typedef int EdgeData;
  typedef int GatherResult;
  static const int gatherZero = INT_MAX;
  static const bool runScatter = true;
  __host__ __device__ static int gatherReduce(const int &a, const int &b) { return a < b ? a : b; }
  __host__ __device__ static int gatherMap(const int *, const int *src, const int *edge) {
    return *src + *edge;
  }
  __host__ __device__ static bool apply(int *v, int g) {
    if (g < *v) {
      *v = g;
      return true;
    }
    return false;
  }
  __host__ __device__ static void scatter(const int *src, const int *dst, int *edge) {
    *edge += 1 + ((*src + *dst) & 1);
  }
};

int main(int argc, char **argv) {
  if (argc != 3) return 2;
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 2;
  int hdr[2];
  if (fread(hdr, 4, 2, f) != 2) return 2;
  const int nV = hdr[0], nE = hdr[1];
  std::vector<int> src(nE), dst(nE), uses(nE), label(nV);
  if (fread(src.data(), 4, nE, f) != (size_t)nE || fread(dst.data(), 4, nE, f) != (size_t)nE ||
      fread(uses.data(), 4, nE, f) != (size_t)nE)
    return 2;
  fclose(f);
  for (int v = 0; v < nV; ++v) label[v] = 3 * v;
  GASEngineGPU<TAging> engine;
  engine.setGraph(nV, label.data(), nE, uses.data(), src.data(), dst.data());
  engine.setActive(0, nV);
  int iters = 0;
  while (engine.countActive()) {
    engine.gather();
    engine.apply();
    engine.scatterActivate();
    engine.nextIter();
    ++iters;
  }
  engine.getResults();
  FILE *o = fopen(argv[2], "wb");
  if (!o) return 2;
  fwrite(label.data(), 4, nV, o);
  fwrite(uses.data(), 4, nE, o);
  fwrite(&iters, 4, 1, o);
  fclose(o);
  return 0;
}
