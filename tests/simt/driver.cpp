// Runs the engine (built from its CUDA sources for host execution) on one
// dataset: driver X.f32 n d eps F num_obj min_size r cells rect out.bin
// Writes: k, then per clustered subspace |S|, its dims and n labels (int32).
#include <unistd.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "inscy_gb300.h"

namespace simt {
long long launches();
}

int main(int argc, char** argv) {
  if (argc < 12) {
    std::fprintf(stderr, "usage: driver X.f32 n d eps F num_obj min_size r cells rect out.bin [entropy_order]\n");
    return 2;
  }
  const long long n = atoll(argv[2]);
  const int d = atoi(argv[3]);
  std::vector<float> X((size_t)n * d);
  FILE* f = fopen(argv[1], "rb");
  if (!f || fread(X.data(), 4, X.size(), f) != X.size()) {
    std::fprintf(stderr, "cannot read %s\n", argv[1]);
    return 2;
  }
  fclose(f);
  inscy_params p{(float)atof(argv[4]), (float)atof(argv[5]), atoi(argv[6]), atoi(argv[7]), (float)atof(argv[8]),
                 atoi(argv[9]), atoi(argv[10]), argc > 12 ? atoi(argv[12]) : 0};
  inscy_result* r = nullptr;
  if (inscy_run(X.data(), n, d, &p, INSCY_MODE_PLAIN, &r) != INSCY_OK) {
    std::fprintf(stderr, "inscy_run: %s\n", inscy_last_error());
    std::fflush(stderr);
    _exit(1);
  }
  const int k = inscy_result_count(r);
  FILE* o = fopen(argv[11], "wb");
  fwrite(&k, 4, 1, o);
  for (int i = 0; i < k; ++i) {
    int dims[64];
    const int m = inscy_result_subspace(r, i, dims, 64);
    fwrite(&m, 4, 1, o);
    fwrite(dims, 4, m, o);
    fwrite(inscy_result_labels_ptr(r, i), 4, n, o);
  }
  fclose(o);
  std::fprintf(stderr, "%d clustered subspaces, %lld launches\n", k, simt::launches());
  inscy_result_free(r);
  std::fflush(stderr);
  _exit(0);  // the block worker threads stay parked
}
