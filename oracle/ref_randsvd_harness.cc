/*
 * Test infrastructure (oracle): drives the REFERENCE's own randomized SVD,
 * mkl_redsvd::MKLRedSVD<float>::run (LightNE/mklredsvd/mklredsvd.cc:93-403,
 * with util.cc's gram_schmidt), followed by path_embed::compute_u_sigma_root
 * (LightNE/PathEmbed.h:371-408), compiled from the reference sources where
 * they lie, so that its outputs can pin the FP64 restatement in
 * oracle/linalg_oracle.py and the golden fixtures under tests/golden/.
 * Nothing in the product links or runs this program.
 *
 *   ref_randsvd <a.csr> <omega.f32> <p.f32> <out.bin> rank dim normalize
 *
 * The CSR file is the "LNECSR01" format of lightne_gb300/graphs.py.  MKL is
 * not available here, so the routines run() calls come from
 * oracle/mkl_shim/mkl_defs.h; its Gaussian stream returns the queued Omega
 * (n x rank) and then P (rank x rank), the sketches the reference draws from
 * VSL's SFMT19937 stream with seed 777 (which cannot be reproduced without
 * MKL).
 *
 * Output ("LNESVD01", little endian): int64 n, rank, dim; float32 S[rank],
 * matU[n x rank], emb[n x dim].
 */
#include "mkl.h"
#include "mkl_defs.h"
#include "SpectralPropagation.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

static bool read_all(const char* path, std::vector<char>& out) {
  std::FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  out.resize((size_t)sz);
  bool ok = std::fread(out.data(), 1, out.size(), f) == out.size();
  std::fclose(f);
  return ok;
}

int main(int argc, char** argv) {
  if (argc != 8) {
    std::fprintf(stderr, "usage: %s a.csr omega.f32 p.f32 out.bin rank dim normalize\n", argv[0]);
    return 2;
  }
  const MKL_INT rank = std::atoll(argv[5]);
  const size_t dim = std::strtoull(argv[6], nullptr, 10);
  const bool normalize = std::atoi(argv[7]) != 0;
  std::vector<char> raw;
  if (!read_all(argv[1], raw) || raw.size() < 24 || std::memcmp(raw.data(), "LNECSR01", 8) != 0) {
    std::fprintf(stderr, "cannot read %s\n", argv[1]);
    return 1;
  }
  int64_t n, nnz;
  std::memcpy(&n, raw.data() + 8, 8);
  std::memcpy(&nnz, raw.data() + 16, 8);
  std::vector<MKL_INT> rows((size_t)n + 1), col((size_t)nnz);
  std::vector<float> val((size_t)nnz);
  const char* p = raw.data() + 24;
  for (int64_t i = 0; i <= n; ++i) { int64_t v; std::memcpy(&v, p + 8 * i, 8); rows[i] = v; }
  p += 8 * (n + 1);
  for (int64_t i = 0; i < nnz; ++i) { int32_t v; std::memcpy(&v, p + 4 * i, 4); col[i] = v; }
  p += 4 * nnz;
  std::memcpy(val.data(), p, 4 * nnz);
  std::vector<char> om, pm;
  if (!read_all(argv[2], om) || !read_all(argv[3], pm) || om.size() != (size_t)(4 * n * rank) ||
      pm.size() != (size_t)(4 * rank * rank)) {
    std::fprintf(stderr, "sketch files do not hold n x rank and rank x rank floats\n");
    return 1;
  }
  std::vector<float>& q = lne_shim::gaussian_queue();
  q.resize((om.size() + pm.size()) / 4);
  std::memcpy(q.data(), om.data(), om.size());
  std::memcpy(q.data() + om.size() / 4, pm.data(), pm.size());

  mkl_redsvd::MKLRedSVD<float> svd((MKL_INT)n, rows.data(), rows.data() + 1, col.data(), val.data(), false, rank,
                                   false);
  svd.run();
  float* emb = path_embed::compute_u_sigma_root<float>(svd.matU, svd.S, (size_t)n, (size_t)rank, dim, normalize,
                                                       0.0f);
  std::FILE* f = std::fopen(argv[4], "wb");
  if (!f) { std::perror("fopen"); return 1; }
  const int64_t hdr[3] = {n, (int64_t)rank, (int64_t)dim};
  std::fwrite("LNESVD01", 1, 8, f);
  std::fwrite(hdr, 8, 3, f);
  std::fwrite(svd.S, 4, (size_t)rank, f);
  std::fwrite(svd.matU, 4, (size_t)(n * rank), f);
  std::fwrite(emb, 4, (size_t)n * dim, f);
  std::fclose(f);
  delete[] emb;
  return 0;
}
