// Cross-check of the C++ state-file reader/writer (include/imps_io.hpp) with the Python one.
//
//   imps_io_check copy IN OUT   load IN, check that the sector tables and flat buffers give the
//                               tensors back, print a one-line JSON summary (sectors, elements
//                               and an order-sensitive checksum of every flat buffer), save OUT
//   imps_io_check make OUT      write a fixed two-site state whose values are i/64 (exact)
//   imps_io_check alrn IN OUT   load a saveALRN file, print the null spaces' summary, save OUT
//
// Exit status 0 on success; a format error prints it and exits 1.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>

#include "imps_io.hpp"

namespace {

double checksum(const std::vector<double>& v) {
  double s = 0.0;
  for (size_t i = 0; i < v.size(); ++i) s += v[i] * double(i % 7 + 1);
  return s;
}

bool same(const imps_io::mps_tensor& a, const imps_io::mps_tensor& b) {
  if (a.d != b.d || a.blocks.size() != b.blocks.size()) return false;
  for (size_t s = 0; s < a.blocks.size(); ++s) {
    if (a.blocks[s].size() != b.blocks[s].size()) return false;
    for (const auto& kv : a.blocks[s]) {
      auto it = b.blocks[s].find(kv.first);
      if (it == b.blocks[s].end() || it->second.first != kv.second.first ||
          it->second.second.data != kv.second.second.data || it->second.second.rows != kv.second.second.rows)
        return false;
    }
  }
  return true;
}

std::string summary_mps(const std::vector<imps_io::mps_tensor>& v) {
  std::string s = "[";
  for (size_t n = 0; n < v.size(); ++n) {
    auto t = imps_io::mps_table(v[n]);
    auto f = imps_io::flat(v[n]);
    char buf[160];
    std::snprintf(buf, sizeof buf, "%s{\"d\": %u, \"nblocks\": %d, \"nelem\": %zu, \"checksum\": %.17g}",
                  n ? ", " : "", v[n].d, t.nblocks(), f.size(), checksum(f));
    s += buf;
  }
  return s + "]";
}

std::string summary_diag(const std::vector<imps_io::block_diag>& v) {
  std::string s = "[";
  for (size_t n = 0; n < v.size(); ++n) {
    auto f = imps_io::flat(v[n]);
    char buf[128];
    std::snprintf(buf, sizeof buf, "%s{\"nblocks\": %zu, \"nelem\": %zu, \"checksum\": %.17g}", n ? ", " : "",
                  v[n].size(), f.size(), checksum(f));
    s += buf;
  }
  return s + "]";
}

std::string summary_lam(const std::vector<imps_io::block_lam>& v) {
  std::string s = "[";
  for (size_t n = 0; n < v.size(); ++n) {
    std::vector<double> f;
    for (const auto& kv : v[n]) f.insert(f.end(), kv.second.begin(), kv.second.end());
    char buf[128];
    std::snprintf(buf, sizeof buf, "%s{\"nblocks\": %zu, \"nelem\": %zu, \"checksum\": %.17g}", n ? ", " : "",
                  v[n].size(), f.size(), checksum(f));
    s += buf;
  }
  return s + "]";
}

imps_io::dense fill(uint64_t r, uint64_t c, double& next) {
  imps_io::dense m;
  m.rows = r;
  m.cols = c;
  for (uint64_t i = 0; i < r * c; ++i) m.data.push_back((next += 1.0) / 64.0);
  return m;
}

imps_io::imps_state make_state() {
  // two sites, d = 2, one U(1) label; bond 0 sectors {-1: 1, 1: 2}, bond 1 sectors {0: 2, 2: 1}
  // site n maps bond n -> bond n + 1 with the label shifted by -1 (s = 0) or +1 (s = 1)
  imps_io::imps_state st;
  double next = 0.0;
  std::map<imps_io::key, int> bond[2] = {{{{-1}, 1}, {{1}, 2}}, {{{0}, 2}, {{2}, 1}}};
  for (int n = 0; n < 2; ++n) {
    imps_io::mps_tensor A;
    A.d = 2;
    A.blocks.resize(2);
    for (int s = 0; s < 2; ++s)
      for (const auto& kv : bond[n]) {
        imps_io::key qo{kv.first[0] + (s ? 1 : -1)};
        auto it = bond[1 - n].find(qo);
        if (it != bond[1 - n].end()) A.blocks[s][kv.first] = {qo, fill(kv.second, it->second, next)};
      }
    st.al.push_back(A);
    st.ar.push_back(A);
    imps_io::block_diag C;
    imps_io::block_lam L;
    for (const auto& kv : bond[1 - n]) {
      C[kv.first] = fill(kv.second, kv.second, next);
      L[kv.first] = fill(kv.second, 1, next).data;
    }
    st.c.push_back(C);
    st.lam.push_back(L);
  }
  return st;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    std::string mode = argc > 1 ? argv[1] : "";
    if (mode == "alrn" && argc == 4) {  // loadALRN and saveALRN of the excitation driver's file
      std::ifstream in(argv[2], std::ios::binary);
      imps_io::alrn_state st = imps_io::load_alrn(in);
      std::printf("{\"sites\": %zu, \"nl\": %s}\n", st.al.size(), summary_mps(st.nl).c_str());
      std::ofstream f(argv[3], std::ios::binary);
      imps_io::save(f, st);
      return f.good() ? 0 : 1;
    }
    if (mode == "make" && argc == 3) {
      std::ofstream f(argv[2], std::ios::binary);
      imps_io::save(f, make_state());
      return f.good() ? 0 : 1;
    }
    if (mode != "copy" || argc != 4) {
      std::fprintf(stderr, "usage: %s copy IN OUT | make OUT | alrn IN OUT\n", argv[0]);
      return 2;
    }
    imps_io::imps_state st = imps_io::load_imps(argv[2]);
    for (const auto* arr : {&st.al, &st.ar})
      for (const auto& A : *arr)
        if (!same(imps_io::mps_from_flat(imps_io::mps_table(A), A.d, imps_io::flat(A)), A)) {
          std::fprintf(stderr, "table / flat round trip failed\n");
          return 1;
        }
    for (const auto& C : st.c)
      if (imps_io::diag_from_flat(imps_io::diag_table(C), imps_io::flat(C)).size() != C.size()) return 1;
    std::printf("{\"sites\": %zu, \"lam\": %s, \"c\": %s, \"al\": %s, \"ar\": %s}\n", st.al.size(),
                summary_lam(st.lam).c_str(), summary_diag(st.c).c_str(), summary_mps(st.al).c_str(),
                summary_mps(st.ar).c_str());
    std::ofstream f(argv[3], std::ios::binary);
    imps_io::save(f, st);
    return f.good() ? 0 : 1;
  } catch (const imps_io::format_error& e) {
    std::fprintf(stderr, "format error: %s\n", e.what());
    return 1;
  }
}
