/*
 * Test infrastructure (oracle): drives the REFERENCE's own spectral
 * propagation, spectral_propagation::chebyshev_expansion<Graph, float>
 * (LightNE/SpectralPropagation.h:45-229), compiled from its sources where
 * they lie, so that its outputs can pin the FP64 restatement in
 * oracle/linalg_oracle.py and the golden fixtures under tests/golden/.
 * Nothing in the product links or runs this program.
 *
 *   ref_propagate <graph.adj> <a.f32> <out.bin> dim order mu s
 *
 * It reads the AdjacencyGraph text with the reference reader
 * (ligra/graph_io.h:185-250) and the n x dim float32 input embedding a, and
 * calls chebyshev_expansion(a, G, dim, dim, order, mu, s), the call of
 * LightNE.cc:114 (rank == dim).  The MKL and Boost routines it needs come
 * from oracle/mkl_shim/mkl_defs.h and oracle/boost_shim (MKL and Boost are
 * not available here); the SVD stand-in records the matrix the reference
 * passes to get_embedding_dense.
 *
 * Output ("LNEPRP01", little endian): int64 n, int64 dim, then three
 * float32 n x dim matrices: a after the call (a - conv: the reference
 * mutates its argument), the (A + I)(a - conv) product handed to
 * get_embedding_dense, and the returned embedding.
 */
#include "mkl.h"
#include "mkl_defs.h"
#include "SpectralPropagation.h"

#include <cstdio>
#include <cstdlib>
#include <vector>

int main(int argc, char** argv) {
  if (argc != 8) {
    std::fprintf(stderr, "usage: %s graph.adj a.f32 out.bin dim order mu s\n", argv[0]);
    return 2;
  }
  auto G = gbbs_io::read_unweighted_symmetric_graph(argv[1], false);
  const int64_t n = (int64_t)G.n;
  const int64_t dim = std::atoll(argv[4]);
  const size_t order = std::strtoull(argv[5], nullptr, 10);
  const float mu = (float)std::strtod(argv[6], nullptr);
  const float s = (float)std::strtod(argv[7], nullptr);
  std::vector<float> a((size_t)(n * dim));
  std::FILE* fa = std::fopen(argv[2], "rb");
  if (!fa || std::fread(a.data(), 4, a.size(), fa) != a.size()) {
    std::fprintf(stderr, "cannot read %s\n", argv[2]);
    return 1;
  }
  std::fclose(fa);
  float* emb = spectral_propagation::chebyshev_expansion<decltype(G), float>(a.data(), G, (MKL_INT)dim,
                                                                             (MKL_INT)dim, order, mu, s);
  const std::vector<double>& y = lne_shim::last_svd_input();
  if ((int64_t)y.size() != n * dim) {
    std::fprintf(stderr, "the SVD stand-in saw no n x dim input\n");
    return 1;
  }
  std::vector<float> yf(y.begin(), y.end());
  std::FILE* f = std::fopen(argv[3], "wb");
  if (!f) { std::perror("fopen"); return 1; }
  std::fwrite("LNEPRP01", 1, 8, f);
  std::fwrite(&n, 8, 1, f);
  std::fwrite(&dim, 8, 1, f);
  std::fwrite(a.data(), 4, a.size(), f);
  std::fwrite(yf.data(), 4, yf.size(), f);
  std::fwrite(emb, 4, (size_t)(n * dim), f);
  std::fclose(f);
  delete[] emb;
  return 0;
}
