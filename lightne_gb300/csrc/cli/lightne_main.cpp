// LightNE — drop-in command line for the reference binary (LightNE/LightNE.cc)
// on top of liblightne_gb300.so.
//
//   LightNE [flags] <graph.adj>
//
// Same flags, input and outputs as the reference: the AdjacencyGraph text
// file is the last argument (ligra/parse_command_line.h: getArgument(0)),
// flags are matched as exact tokens with the value in the next token
// (getOptionLongValue / getOptionDoubleValue / getOptionValue), -ne_out and
// -pro_out receive raw little-endian float32 n x dim row-major matrices with
// no header (LightNE.cc:18-27), and the "###" parameter banner and
// "### Running Time" lines are printed as LightNE.cc:64-120 prints them.
//
// Added flags (defaults keep the reference behaviour): -seed <u64> (the
// reference seeds the sampler with time(0), PathEmbed.h:499), -mu and
// -theta (hard-coded 0.2 and 0.5 at LightNE.cc:114), -precision
// fp32|bf16|fp16 (SpMM dense operand; default fp32), -device <int>.
//
// Exit status: 0 on success; the library's status code (with its message on
// stderr) on failure.  Where the reference prints "looping forever" and
// exits 0 on a full pair table (LightNE/par_table.h:104-107), this program
// prints the same line and exits with LNE_ERR_TABLE_FULL.
#include <errno.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>

#include <chrono>
#include <sstream>
#include <string>
#include <vector>

#include "lightne_gb300.h"

namespace {

struct CommandLine {
  int argc;
  char** argv;
  std::string getArgument(int i) const { return argc >= 2 + i ? std::string(argv[argc - 1 - i]) : std::string(); }
  const char* value(const char* opt) const {
    for (int i = 1; i < argc - 1; ++i)
      if (strcmp(argv[i], opt) == 0) return argv[i + 1];
    return nullptr;
  }
  bool present(const char* opt) const {
    for (int i = 1; i < argc; ++i)
      if (strcmp(argv[i], opt) == 0) return true;
    return false;
  }
  long getLong(const char* opt, long def) const {
    const char* v = value(opt);
    return v ? atol(v) : def;
  }
  double getDouble(const char* opt, double def) const {
    const char* v = value(opt);
    double d;
    if (!v) return def;
    if (sscanf(v, "%lf", &d) == EOF) {
      fprintf(stderr, "usage: %s [flags] <inFile>\n", argv[0]);
      exit(2);
    }
    return d;
  }
  std::string getString(const char* opt, const char* def) const {
    const char* v = value(opt);
    return v ? std::string(v) : std::string(def);
  }
};

double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// AdjacencyGraph text: "AdjacencyGraph", n, m, n offsets, m targets
// (ligra/graph_io.h:185-230).  Returns false with a message on error.
bool read_adjacency_graph(const std::string& path, std::vector<int64_t>& off, std::vector<int32_t>& nbrs,
                          std::string& err) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) {
    err = path + ": " + strerror(errno);
    return false;
  }
  struct stat sb;
  fstat(fileno(f), &sb);
  std::vector<char> buf((size_t)sb.st_size + 1);
  size_t got = fread(buf.data(), 1, (size_t)sb.st_size, f);
  fclose(f);
  buf[got] = '\0';
  const char* p = buf.data();
  const char* end = p + got;
  // Binary AdjacencyGraph ("LNEADJ01", int64 n, int64 m, int64 offsets[n + 1],
  // int32 targets[m], little endian), written by lightne_gb300.x2adj and
  // graphs.write_adjacency_binary: the same arrays without text parsing.
  if (got >= 24 && memcmp(p, "LNEADJ01", 8) == 0) {
    int64_t n = 0, m = 0;
    memcpy(&n, p + 8, 8);
    memcpy(&m, p + 16, 8);
    if (n < 0 || m < 0 || (uint64_t)got != 24 + 8 * (uint64_t)(n + 1) + 4 * (uint64_t)m) {
      err = path + ": bad binary AdjacencyGraph size";
      return false;
    }
    off.resize((size_t)n + 1);
    nbrs.resize((size_t)m);
    memcpy(off.data(), p + 24, 8 * (size_t)(n + 1));
    memcpy(nbrs.data(), p + 24 + 8 * (size_t)(n + 1), 4 * (size_t)m);
    if (off[0] != 0 || off[n] != m) {
      err = path + ": binary AdjacencyGraph offsets do not span the targets";
      return false;
    }
    return true;
  }
  auto skip = [&]() { while (p < end && (*p == ' ' || *p == '\n' || *p == '\t' || *p == '\r')) ++p; };
  auto next_u64 = [&](uint64_t& v) -> bool {
    skip();
    if (p >= end || *p < '0' || *p > '9') return false;
    v = 0;
    while (p < end && *p >= '0' && *p <= '9') v = v * 10 + (uint64_t)(*p++ - '0');
    return true;
  };
  skip();
  if (end - p < 14 || strncmp(p, "AdjacencyGraph", 14) != 0) {
    err = path + ": not an AdjacencyGraph file";
    return false;
  }
  p += 14;
  uint64_t n, m;
  if (!next_u64(n) || !next_u64(m)) {
    err = path + ": bad header";
    return false;
  }
  off.resize(n + 1);
  nbrs.resize(m);
  for (uint64_t i = 0; i < n; ++i) {
    uint64_t v;
    if (!next_u64(v)) { err = path + ": truncated offsets"; return false; }
    off[i] = (int64_t)v;
  }
  off[n] = (int64_t)m;
  for (uint64_t i = 0; i < m; ++i) {
    uint64_t v;
    if (!next_u64(v)) { err = path + ": truncated edges"; return false; }
    nbrs[i] = (int32_t)v;
  }
  return true;
}

int fail(int rc, const char* where) {
  fprintf(stderr, "LightNE: %s failed (status %d): %s\n", where, rc, lne_last_error());
  return rc;
}

void save(const std::string& file, const std::vector<float>& emb) {
  const double t0 = now();
  if (FILE* f = fopen(file.c_str(), "wb")) {
    fwrite(emb.data(), sizeof(float), emb.size(), f);
    fclose(f);
  }
  printf("PBBS-time: save time: %.4f\n", now() - t0);
}

}  // namespace

int main(int argc, char** argv) {
  CommandLine P{argc, argv};
  if (argc < 2) {
    fprintf(stderr, "usage: %s [-s] <inFile>\n", argv[0]);
    return 2;
  }
  const std::string iFile = P.getArgument(0);
  if (!P.present("-s")) {
    printf("# The application expects the input graph to be symmetric (-s flag).\n");
    printf("# Please run on a symmetric input.\n");
  }
  if (P.present("-c")) {
    fprintf(stderr, "LightNE: compressed graph input (-c) is not supported by this build\n");
    return LNE_ERR_UNSUPPORTED;
  }
  const long rounds = P.getLong("-rounds", 3);
  const long walks_per_edge = P.getLong("-walksperedge", 100);
  const long walk_len = P.getLong("-walklen", 10);
  const long table_size = P.getLong("-tablesz", 0);
  const long rank = P.getLong("-rank", 256);
  const long dim = P.getLong("-dim", 128);
  const long order = P.getLong("-order", 10);
  const long negative = P.getLong("-negative", 1);
  const bool upper = P.getLong("-upper", 0) != 0;
  const bool sample = P.getLong("-sample", 0) != 0;
  const bool analyze = P.getLong("-analyze", 0) != 0;
  const bool normalize = P.getLong("-normalize", 0) != 0;
  const float sample_ratio = (float)P.getDouble("-sample_ratio", 1.0);
  const float mem_ratio = (float)P.getDouble("-mem_ratio", 1.0);
  const std::string ne_method = P.getString("-ne_method", "netsmf");
  const std::string ne_out = P.getString("-ne_out", "");
  const std::string pro_out = P.getString("-pro_out", "");
  const std::string step_coeff_str = P.getString("-step_coeff", "1,1,1,1,1,1,1,1,1,1");
  const bool random_project_only = P.getLong("-random_project_only", 0) != 0;
  const bool sparse_project = P.getLong("-sparse_project", 0) != 0;
  const float sparse_project_s = (float)P.getDouble("-sparse_project_s", 100.0);
  const double mu = P.getDouble("-mu", 0.2);
  const double theta = P.getDouble("-theta", 0.5);
  const std::string precision = P.getString("-precision", "fp32");
  const int device = (int)P.getLong("-device", 0);
  const char* seed_s = P.value("-seed");

  std::vector<float> step_coeff;
  {
    std::stringstream ss(step_coeff_str);
    while (ss.good()) {
      std::string sub;
      std::getline(ss, sub, ',');
      step_coeff.push_back(std::stof(sub));
    }
  }
  if (ne_method != "netsmf" && ne_method != "ne_zhang_et_al") {
    fprintf(stderr, "LightNE: -ne_method must be netsmf or ne_zhang_et_al\n");
    return LNE_ERR_INVALID;
  }
  if ((long)step_coeff.size() != walk_len) {
    fprintf(stderr, "LightNE: -step_coeff must have -walklen entries\n");
    return LNE_ERR_INVALID;
  }
  if (precision != "fp32" && precision != "bf16" && precision != "fp16") {
    fprintf(stderr, "LightNE: -precision must be fp32, bf16 or fp16\n");
    return LNE_ERR_INVALID;
  }
  const int prec = precision == "bf16" ? LNE_PREC_BF16 : (precision == "fp16" ? LNE_PREC_FP16 : LNE_PREC_FP32);

  std::vector<int64_t> off;
  std::vector<int32_t> nbrs;
  std::string err;
  if (!read_adjacency_graph(iFile, off, nbrs, err)) {
    fprintf(stderr, "LightNE: %s\n", err.c_str());
    return LNE_ERR_INVALID;
  }
  const int64_t n = (int64_t)off.size() - 1, m = off[n];

  lne_ctx* ctx = nullptr;
  int rc;
  if ((rc = lne_ctx_create(&ctx, device, nullptr))) return fail(rc, "lne_ctx_create");
  lne_graph* g = nullptr;
  if ((rc = lne_graph_upload(ctx, n, off.data(), nbrs.data(), &g))) return fail(rc, "lne_graph_upload");

  double total_time = 0.0;
  for (long round = 0; round < rounds; ++round) {
    printf("### Application: LightNE_mkl\n");
    printf("### Graph: %s\n", iFile.c_str());
    printf("### Threads: %d\n", 1);
    printf("### n: %lld\n", (long long)n);
    printf("### m: %lld\n", (long long)m);
    printf("### Params: \n");
    printf("###  -walksperedge = %ld\n", walks_per_edge);
    printf("###  -walklen = %ld\n", walk_len);
    printf("###  -tablesz = %ld\n", table_size);
    printf("###  -rank = %ld\n", rank);
    printf("###  -dim = %ld\n", dim);
    printf("###  -order = %ld\n", order);
    printf("###  -negative = %ld\n", negative);
    printf("###  -upper = %s\n", upper ? "true" : "false");
    printf("###  -sample = %s\n", sample ? "true" : "false");
    printf("###  -analyze = %s\n", analyze ? "true" : "false");
    printf("###  -ne_method = %s (nestmf: see Qiu etal: arxiv.org/abs/1906.11156, ne_zhang_et_al: see sec. 3.1 "
           "of Zhang et al: www.ijcai.org/proceedings/2019/594)\n", ne_method.c_str());
    printf("###  -normalize = %d\n", normalize ? 1 : 0);
    printf("###  -sample_ratio = %g\n", sample_ratio);
    printf("###  -mem_ratio = %g\n", mem_ratio);
    printf("###  -random_project_only = %d\n", random_project_only ? 1 : 0);
    printf("###  -sparse_project = %d\n", sparse_project ? 1 : 0);
    printf("###  -sparse_project_s = %g\n", sparse_project_s);
    printf("###  -ne_out = %s\n", ne_out.c_str());
    printf("###  -pro_out = %s\n", pro_out.c_str());
    printf("###  -step_coeff = ");
    for (float c : step_coeff) printf("%g ", c);
    printf("\n### ------------------------------------\n");
    fflush(stdout);
    const double t0 = now();

    lne_csr* csr = nullptr;
    const bool zhang = ne_method == "ne_zhang_et_al";
    if (zhang) {
      // NE_Zhang_et_al (PathEmbed.h:410-463): the 1-hop log matrix, then the
      // same SVD with normalised rows
      if ((rc = lne_ne_zhang_matrix(ctx, g, &csr))) return fail(rc, "lne_ne_zhang_matrix");
    } else {
      const uint64_t seed = seed_s ? strtoull(seed_s, nullptr, 10) : (uint64_t)time(nullptr);
      printf("# seed = %llu\n", (unsigned long long)seed);
      lne_sparsify_params sp = {seed, walk_len, table_size, negative, sample ? 1 : 0, 0, sample_ratio, mem_ratio};
      // -upper keeps only the upper triangle for MKL's symmetric descriptor;
      // the matrix is the same, so the full symmetric CSR is built for the SVD.
      lne_sparsify_stats st;
      if ((rc = lne_sparsify(ctx, g, &sp, &csr, &st))) {
        if (rc == LNE_ERR_TABLE_FULL) printf("looping forever\n");
        return fail(rc, "lne_sparsify");
      }
      printf("# logn = %g sample_ratio = %g mem_ratio = %g\n", st.logn, sample_ratio, mem_ratio);
      printf("# table_size = %lld\n# actual table.size = %lld\n", (long long)st.table_size, (long long)st.capacity);
      printf("# total samples = %g\n# 1/lambda = %g\n# exp_rv_rounded = %lld\n# fractional_bits = %g\n",
             st.total_samples, st.inv_lambda, (long long)st.exp_rv_rounded, st.frac);
      printf("PBBS-time: # count time: %.4f\n", st.ms_sample / 1e3);
      printf("# tot wgh (samples) = %g\n# factor = %g\n", st.m_exact, st.factor);
      printf("# nnz in upper triangle of sparsifier = %lld\n# nnz in sparsifier = %lld\n", (long long)st.nnz_upper,
             (long long)st.nnz);
      printf("PBBS-time: # generate matrix time: %.4f\n", (st.ms_sample + st.ms_trunclog + st.ms_csr) / 1e3);
    }

    float* d_emb = nullptr;
    if ((rc = lne_device_alloc(ctx, (int64_t)sizeof(float) * n * dim, (void**)&d_emb)))
      return fail(rc, "lne_device_alloc");
    std::vector<float> S(rank);
    lne_randsvd_params rp = {rank, dim, (normalize || zhang) ? 1 : 0, prec, 777, (random_project_only && !zhang) ? 1 : 0,
                             (sparse_project && !zhang) ? 1 : 0, (double)sparse_project_s};
    lne_randsvd_stats rs;
    if ((rc = lne_randsvd(ctx, csr, &rp, d_emb, S.data(), &rs))) return fail(rc, "lne_randsvd");
    lne_csr_free(csr);
    if (!random_project_only)
      printf("# computing u*sqrt(sigma), sigma(0)=%g, sigma(%ld)=%g\n", S[0], dim - 1, S[dim - 1]);
    printf("PBBS-time: # svd time: %.4f\n", rs.ms_total / 1e3);
    std::vector<float> emb((size_t)n * dim);
    if ((rc = lne_copy_to_host(ctx, emb.data(), d_emb, (int64_t)sizeof(float) * n * dim)))
      return fail(rc, "lne_copy_to_host");
    if (!ne_out.empty()) {
      printf("dump network embedding to %s\n", ne_out.c_str());
      save(ne_out, emb);
    }
    if (!pro_out.empty()) {
      const double tp = now();
      float *d_y = nullptr, *d_pro = nullptr;
      if ((rc = lne_device_alloc(ctx, (int64_t)sizeof(float) * n * dim, (void**)&d_y)) ||
          (rc = lne_device_alloc(ctx, (int64_t)sizeof(float) * n * dim, (void**)&d_pro)))
        return fail(rc, "lne_device_alloc");
      lne_propagate_params pp = {dim, (int32_t)order, prec, mu, theta};
      lne_propagate_stats ps;
      if ((rc = lne_propagate(ctx, g, &pp, d_emb, d_y, nullptr, &ps))) return fail(rc, "lne_propagate");
      if ((rc = lne_dense_embed(ctx, d_y, n, dim, d_pro, nullptr))) return fail(rc, "lne_dense_embed");
      std::vector<float> pro((size_t)n * dim);
      if ((rc = lne_copy_to_host(ctx, pro.data(), d_pro, (int64_t)sizeof(float) * n * dim)))
        return fail(rc, "lne_copy_to_host");
      lne_device_free(ctx, d_y);
      lne_device_free(ctx, d_pro);
      printf("PBBS-time: proX time: %.4f\n", now() - tp);
      printf("dump proX embedding to %s\n", pro_out.c_str());
      save(pro_out, pro);
    }
    lne_device_free(ctx, d_emb);
    const double tt = now() - t0;
    printf("### Running Time: %g\n", tt);
    fflush(stdout);
    total_time += tt;
  }
  printf("# time per iter: %g\n", total_time / (rounds > 0 ? rounds : 1));
  lne_graph_free(g);
  lne_ctx_destroy(ctx);
  return 0;
}
