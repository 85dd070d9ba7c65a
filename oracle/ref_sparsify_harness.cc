/*
 * Test infrastructure (oracle): drives the REFERENCE's own sparsifier,
 * compiled from its sources where they lie, so that its output can pin the
 * CPU restatement in oracle/sparsify_port.c and the golden fixtures under
 * tests/golden/.  Nothing in the product links or runs this program.
 *
 *   ref_sparsify <graph.adj> <out.csr> seed walk_len tablesz negative sample
 *                sample_ratio mem_ratio upper
 *
 * It reads the AdjacencyGraph text with the reference reader
 * (ligra/graph_io.h:185-250), calls
 * path_embed::generate_trunc_log_matrix_v2<Graph,float>
 * (LightNE/PathEmbed.h:81-369) with an explicit pbbs::random(seed) in place
 * of the time(0) seed of LightNE/PathEmbed.h:499, and writes the CSR in
 * canonical form: each row sorted by column.  The reference scatters a row's
 * entries in a nondeterministic order (LightNE/PathEmbed.h:300-311); the set
 * of (col, value) pairs of a row is deterministic, so sorting gives a
 * reproducible image of the reference result.
 *
 * Output file ("LNECSR01"): int64 n, int64 nnz, int64 row_ptr[n+1],
 * int32 col[nnz], float val[nnz] (little endian).  The wall time of the call
 * is printed as "# ref_sparsify seconds = <t>".
 */
#include "PathEmbed.h"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <vector>
#include <algorithm>

int main(int argc, char** argv) {
  if (argc != 11) {
    std::fprintf(stderr, "usage: %s graph.adj out.csr seed walk_len tablesz negative "
                 "sample sample_ratio mem_ratio upper\n", argv[0]);
    return 2;
  }
  const char* gfile = argv[1];
  const char* ofile = argv[2];
  size_t seed = std::strtoull(argv[3], nullptr, 10);
  size_t walk_len = std::strtoull(argv[4], nullptr, 10);
  size_t tablesz = std::strtoull(argv[5], nullptr, 10);
  size_t negative = std::strtoull(argv[6], nullptr, 10);
  bool sample = std::atoi(argv[7]) != 0;
  /* LightNE.cc:42-43 narrows both ratios to float */
  float sample_ratio = static_cast<float>(std::strtod(argv[8], nullptr));
  float mem_ratio = static_cast<float>(std::strtod(argv[9], nullptr));
  bool upper = std::atoi(argv[10]) != 0;

  auto G = gbbs_io::read_unweighted_symmetric_graph(const_cast<char*>(gfile), false);
  std::vector<float> step_coeff(walk_len, 1.0f);

  MKL_INT* rows_start = new MKL_INT[G.n + 1];
  MKL_INT* col_idx = nullptr;
  float* value = nullptr;
  auto t0 = std::chrono::steady_clock::now();
  auto fake = path_embed::generate_trunc_log_matrix_v2<decltype(G), float>(
      G, pbbs::random(seed), /*walks_per_edge=*/1, walk_len, upper, sample, tablesz,
      negative, sample_ratio, mem_ratio, step_coeff, rows_start, col_idx, value);
  auto t1 = std::chrono::steady_clock::now();
  std::printf("# ref_sparsify seconds = %.6f\n",
              std::chrono::duration<double>(t1 - t0).count());

  int64_t n = static_cast<int64_t>(G.n);
  int64_t nnz = static_cast<int64_t>(rows_start[G.n]);
  std::vector<int32_t> col(nnz);
  std::vector<float> val(nnz);
  std::vector<std::pair<int64_t, float>> row;
  for (int64_t i = 0; i < n; ++i) {
    row.clear();
    for (int64_t j = rows_start[i]; j < rows_start[i + 1]; ++j)
      row.emplace_back(col_idx[j], value[j]);
    std::sort(row.begin(), row.end(),
              [](const std::pair<int64_t, float>& a, const std::pair<int64_t, float>& b) {
                return a.first < b.first;
              });
    for (size_t k = 0; k < row.size(); ++k) {
      col[rows_start[i] + k] = static_cast<int32_t>(row[k].first);
      val[rows_start[i] + k] = row[k].second;
    }
  }
  std::FILE* f = std::fopen(ofile, "wb");
  if (!f) { std::perror("fopen"); return 1; }
  std::fwrite("LNECSR01", 1, 8, f);
  std::fwrite(&n, 8, 1, f);
  std::fwrite(&nnz, 8, 1, f);
  std::vector<int64_t> rp(rows_start, rows_start + n + 1);
  std::fwrite(rp.data(), 8, n + 1, f);
  std::fwrite(col.data(), 4, nnz, f);
  std::fwrite(val.data(), 4, nnz, f);
  std::fclose(f);
  return 0;
}
