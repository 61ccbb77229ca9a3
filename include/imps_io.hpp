// State files of the reference (saveIMPS / loadIMPS, MPSBlockUtilities.hpp:1215-1327, and the
// excitation driver's saveALRN / loadALRN, Excitations_helpers.hpp:949-1085) for C++
// host programs: header-only C++17, independent of the GPU library, so that a host can read a
// state the reference wrote, hand its sector tables to imps_layout_create and its flat
// Vectorize buffers to the plans, and write results back in the same format.
//
// File = BLOCKLAMARRAY, RBLOCKDIAGMATARRAY, RBLOCKMPSARRAY (AL), RBLOCKMPSARRAY (AR).  Each
// object: its type name and '\n' (GetHeader, BlockObj.hpp:3156-3192, MPSBlockMat.hpp:1418-1430),
// a 4-byte unsigned count, then its parts:
//   array types         count = sites; the objects (BlockObj.hpp:2692-2708, 2877-2893,
//                       MPSBlockMat.hpp:1326-1342)
//   BLOCKLAM            count = sectors; per sector key, armadillo column (BlockObj.hpp:150-183)
//   RBLOCKDIAGMAT       count = sectors; per sector key, armadillo matrix (BlockObj.hpp:1968-2000)
//   RBLOCKMAT           count = sectors; per sector in key, out key, matrix (BlockObj.hpp:905-945)
//   RBLOCKMPS           d and NSites (4-byte unsigned each), then d^NSites RBLOCKMAT
//                       (MPSBlockMat.hpp:1085-1104)
// key = 4-byte unsigned Nsym + Nsym 4-byte signed labels (KeyTypes.hpp:94-117); sectors in
// std::map order (lexicographic integer vectors).  Dense blocks in armadillo's arma_binary form
// (armadillo is a third-party dependency of the reference, version not pinned there):
// "ARMA_MAT_BIN_FN008\n", "<rows> <cols>\n", rows*cols doubles column-major.  Integers and
// doubles are little-endian (the byte order of both hosts the reference and this code run on).
// Reading uses the reference's stream operations: operator>> for type names and sizes, then
// get() for the one newline after them.
//
// Errors throw imps_io::format_error (the reference's loaders print and return false, and its
// Excitations driver then throws, Excitations_main.cpp:89).
#pragma once

#include <cstdint>
#include <cstring>
#include <fstream>
#include <istream>
#include <map>
#include <ostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace imps_io {

using key = std::vector<int32_t>;

struct dense {  // column-major, as armadillo stores it
  uint64_t rows = 0, cols = 0;
  std::vector<double> data;
};

using block_lam = std::map<key, std::vector<double>>;          // BlockLam
using block_diag = std::map<key, dense>;                        // BlockDiagMat
using block_mat = std::map<key, std::pair<key, dense>>;         // BlockMat: qin -> (qout, block)

struct mps_tensor {  // MPSBlockMat: one BlockMat per physical index
  uint32_t d = 0, nsites = 1;
  std::vector<block_mat> blocks;
};

struct imps_state {  // indexed by site n; c[n] is the centre matrix right of site n
  std::vector<block_lam> lam;
  std::vector<block_diag> c;
  std::vector<mps_tensor> al, ar;
};

struct format_error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

constexpr const char* kLam = "BLOCKLAM";
constexpr const char* kLamArray = "BLOCKLAMARRAY";
constexpr const char* kDiag = "RBLOCKDIAGMAT";
constexpr const char* kDiagArray = "RBLOCKDIAGMATARRAY";
constexpr const char* kMat = "RBLOCKMAT";
constexpr const char* kMps = "RBLOCKMPS";
constexpr const char* kMpsArray = "RBLOCKMPSARRAY";
constexpr const char* kArmaF64 = "ARMA_MAT_BIN_FN008";

namespace detail {

inline void put_u32(std::ostream& os, uint32_t x) {
  unsigned char b[4] = {(unsigned char)(x & 0xff), (unsigned char)((x >> 8) & 0xff),
                        (unsigned char)((x >> 16) & 0xff), (unsigned char)((x >> 24) & 0xff)};
  os.write(reinterpret_cast<const char*>(b), 4);
}

inline void put_f64(std::ostream& os, double v) {
  uint64_t u;
  std::memcpy(&u, &v, 8);
  unsigned char b[8];
  for (int i = 0; i < 8; ++i) b[i] = (unsigned char)((u >> (8 * i)) & 0xff);
  os.write(reinterpret_cast<const char*>(b), 8);
}

inline uint32_t get_u32(std::istream& is) {
  unsigned char b[4];
  if (!is.read(reinterpret_cast<char*>(b), 4)) throw format_error("unexpected end of file");
  return uint32_t(b[0]) | (uint32_t(b[1]) << 8) | (uint32_t(b[2]) << 16) | (uint32_t(b[3]) << 24);
}

inline double get_f64(std::istream& is) {
  unsigned char b[8];
  if (!is.read(reinterpret_cast<char*>(b), 8)) throw format_error("unexpected end of file");
  uint64_t u = 0;
  for (int i = 0; i < 8; ++i) u |= uint64_t(b[i]) << (8 * i);
  double v;
  std::memcpy(&v, &u, 8);
  return v;
}

inline void put_header(std::ostream& os, const char* name) { os << name << '\n'; }

inline void get_header(std::istream& is, const char* expected) {
  std::string h;
  if (!(is >> h)) throw format_error("unexpected end of file");
  is.get();
  if (h != expected) throw format_error("wrong header " + h + ", should be " + expected);
}

inline void put_key(std::ostream& os, const key& k) {
  put_u32(os, uint32_t(k.size()));
  for (int32_t x : k) put_u32(os, uint32_t(x));
}

inline key get_key(std::istream& is) {
  uint32_t n = get_u32(is);
  if (n > 64) throw format_error("key with " + std::to_string(n) + " labels");
  key k(n);
  for (uint32_t i = 0; i < n; ++i) k[i] = int32_t(get_u32(is));
  return k;
}

inline void put_dense(std::ostream& os, const dense& m) {
  if (m.data.size() != m.rows * m.cols) throw format_error("dense block size does not match rows * cols");
  os << kArmaF64 << '\n' << m.rows << ' ' << m.cols << '\n';
  for (double v : m.data) put_f64(os, v);
}

inline dense get_dense(std::istream& is) {
  std::string h;
  dense m;
  if (!(is >> h >> m.rows >> m.cols)) throw format_error("bad armadillo matrix header");
  if (h != kArmaF64) throw format_error("armadillo matrix header " + h + ", should be " + kArmaF64);
  is.get();
  if (m.rows * m.cols > (uint64_t(1) << 34)) throw format_error("armadillo matrix too large");
  m.data.resize(m.rows * m.cols);
  for (auto& v : m.data) v = get_f64(is);
  return m;
}

}  // namespace detail

// ---- one object each ------------------------------------------------------------------------
inline void save(std::ostream& os, const block_lam& L) {
  detail::put_header(os, kLam);
  detail::put_u32(os, uint32_t(L.size()));
  for (const auto& kv : L) {
    detail::put_key(os, kv.first);
    detail::put_dense(os, dense{kv.second.size(), 1, kv.second});
  }
}

inline void save(std::ostream& os, const block_diag& C) {
  detail::put_header(os, kDiag);
  detail::put_u32(os, uint32_t(C.size()));
  for (const auto& kv : C) {
    detail::put_key(os, kv.first);
    detail::put_dense(os, kv.second);
  }
}

inline void save(std::ostream& os, const block_mat& M) {
  detail::put_header(os, kMat);
  detail::put_u32(os, uint32_t(M.size()));
  for (const auto& kv : M) {
    detail::put_key(os, kv.first);
    detail::put_key(os, kv.second.first);
    detail::put_dense(os, kv.second.second);
  }
}

inline void save(std::ostream& os, const mps_tensor& A) {
  uint64_t n = 1;
  for (uint32_t i = 0; i < A.nsites; ++i) n *= A.d;
  if (A.blocks.size() != n) throw format_error("MPS tensor: blocks.size() != d^nsites");
  detail::put_header(os, kMps);
  detail::put_u32(os, A.d);
  detail::put_u32(os, A.nsites);
  for (const auto& bm : A.blocks) save(os, bm);
}

inline block_lam load_lam(std::istream& is) {
  detail::get_header(is, kLam);
  block_lam L;
  for (uint32_t i = 0, n = detail::get_u32(is); i < n; ++i) {
    key k = detail::get_key(is);
    L[k] = detail::get_dense(is).data;
  }
  return L;
}

inline block_diag load_diag(std::istream& is) {
  detail::get_header(is, kDiag);
  block_diag C;
  for (uint32_t i = 0, n = detail::get_u32(is); i < n; ++i) {
    key k = detail::get_key(is);
    C[k] = detail::get_dense(is);
  }
  return C;
}

inline block_mat load_mat(std::istream& is) {
  detail::get_header(is, kMat);
  block_mat M;
  for (uint32_t i = 0, n = detail::get_u32(is); i < n; ++i) {
    key qin = detail::get_key(is);
    key qout = detail::get_key(is);
    M[qin] = {qout, detail::get_dense(is)};
  }
  return M;
}

inline mps_tensor load_mps(std::istream& is) {
  detail::get_header(is, kMps);
  mps_tensor A;
  A.d = detail::get_u32(is);
  A.nsites = detail::get_u32(is);
  uint64_t n = 1;
  for (uint32_t i = 0; i < A.nsites; ++i) {
    n *= A.d;
    if (n > 4096) throw format_error("MPS tensor with more than 4096 physical indices");
  }
  for (uint64_t s = 0; s < n; ++s) A.blocks.push_back(load_mat(is));
  return A;
}

// ---- the state file ---------------------------------------------------------------------------
template <class T>
inline void save_array(std::ostream& os, const char* header, const std::vector<T>& v) {
  detail::put_header(os, header);
  detail::put_u32(os, uint32_t(v.size()));
  for (const auto& x : v) save(os, x);
}

template <class F>
inline auto load_array(std::istream& is, const char* header, F load_one) {
  detail::get_header(is, header);
  std::vector<decltype(load_one(is))> v;
  for (uint32_t i = 0, n = detail::get_u32(is); i < n; ++i) v.push_back(load_one(is));
  return v;
}

// saveIMPS(Lamvec, Cvec, ALvec, ARvec, file) (MPSBlockUtilities.hpp:1215-1244)
inline void save(std::ostream& os, const imps_state& st) {
  save_array(os, kLamArray, st.lam);
  save_array(os, kDiagArray, st.c);
  save_array(os, kMpsArray, st.al);
  save_array(os, kMpsArray, st.ar);
  if (!os) throw format_error("write failed");
}

// loadIMPS(Lamvec, Cvec, ALvec, ARvec, GroupObj, file) (MPSBlockUtilities.hpp:1271-1300)
inline imps_state load(std::istream& is) {
  imps_state st;
  st.lam = load_array(is, kLamArray, load_lam);
  st.c = load_array(is, kDiagArray, load_diag);
  st.al = load_array(is, kMpsArray, load_mps);
  st.ar = load_array(is, kMpsArray, load_mps);
  return st;
}

// GetUniqueFileName (MPShelpers/src/helpers.cpp:154-161): folder/name.ending, else
// folder/name_v1.ending, folder/name_v2.ending, ...
inline std::string unique_file_name(const std::string& name, const std::string& ending = "bin",
                                    const std::string& folder = ".") {
  auto exists = [](const std::string& p) { std::ifstream f(p); return f.good(); };
  std::string p = folder + "/" + name + "." + ending;
  for (unsigned k = 1; exists(p); ++k) p = folder + "/" + name + "_v" + std::to_string(k) + "." + ending;
  return p;
}

// saveIMPS(..., name, ending) (MPSBlockUtilities.hpp:1249-1267): returns the path written
inline std::string save_imps(const imps_state& st, const std::string& name, const std::string& ending = "bin",
                             const std::string& folder = ".") {
  std::string p = unique_file_name(name, ending, folder);
  std::ofstream f(p, std::ios::binary);
  if (!f) throw format_error("cannot open " + p);
  save(f, st);
  return p;
}

// loadIMPS(..., filename) (MPSBlockUtilities.hpp:1305-1327)
inline imps_state load_imps(const std::string& filename) {
  std::ifstream f(filename, std::ios::binary);
  if (!f) throw format_error("file " + filename + " not found");
  return load(f);
}

// ---- the excitation driver's file (saveALRN / loadALRN, Excitations_helpers.hpp:949-1085) -----
struct alrn_state {  // indexed by site n: c[n] right of site n, l[n] = c^T c, r[n] = c c^T
  std::vector<block_diag> c, l, r;
  std::vector<mps_tensor> al, ar, nl;
};

inline void save(std::ostream& os, const alrn_state& st) {
  save_array(os, kDiagArray, st.c);
  save_array(os, kDiagArray, st.l);
  save_array(os, kDiagArray, st.r);
  save_array(os, kMpsArray, st.al);
  save_array(os, kMpsArray, st.ar);
  save_array(os, kMpsArray, st.nl);
  if (!os) throw format_error("write failed");
}

inline alrn_state load_alrn(std::istream& is) {
  alrn_state st;
  st.c = load_array(is, kDiagArray, load_diag);
  st.l = load_array(is, kDiagArray, load_diag);
  st.r = load_array(is, kDiagArray, load_diag);
  st.al = load_array(is, kMpsArray, load_mps);
  st.ar = load_array(is, kMpsArray, load_mps);
  st.nl = load_array(is, kMpsArray, load_mps);
  return st;
}

// ---- to and from the sector tables and flat buffers of the C ABI ------------------------------
// The arguments of imps_layout_create for an MPS tensor (group = physical index) or a
// block-diagonal matrix (group 0), in Vectorize order: physical index, then key order.
struct table {
  int nsym = 0;
  std::vector<int32_t> qin, qout, rows, cols, group;
  int nblocks() const { return int(rows.size()); }
};

inline void add_row(table& t, int g, const key& qi, const key& qo, uint64_t r, uint64_t c) {
  if (t.rows.empty()) t.nsym = int(qi.size());
  if (int(qi.size()) != t.nsym || int(qo.size()) != t.nsym) throw format_error("keys of different lengths");
  t.qin.insert(t.qin.end(), qi.begin(), qi.end());
  t.qout.insert(t.qout.end(), qo.begin(), qo.end());
  t.rows.push_back(int32_t(r));
  t.cols.push_back(int32_t(c));
  t.group.push_back(g);
}

inline table mps_table(const mps_tensor& A) {
  table t;
  for (size_t s = 0; s < A.blocks.size(); ++s)
    for (const auto& kv : A.blocks[s]) add_row(t, int(s), kv.first, kv.second.first, kv.second.second.rows,
                                               kv.second.second.cols);
  return t;
}

inline table diag_table(const block_diag& C) {
  table t;
  for (const auto& kv : C) add_row(t, 0, kv.first, kv.first, kv.second.rows, kv.second.cols);
  return t;
}

// Vectorize (MPSBlockMat.hpp:448-465, BlockObj.hpp:1360-1467): blocks column-major, concatenated
inline std::vector<double> flat(const mps_tensor& A) {
  std::vector<double> v;
  for (const auto& bm : A.blocks)
    for (const auto& kv : bm) v.insert(v.end(), kv.second.second.data.begin(), kv.second.second.data.end());
  return v;
}

inline std::vector<double> flat(const block_diag& C) {
  std::vector<double> v;
  for (const auto& kv : C) v.insert(v.end(), kv.second.data.begin(), kv.second.data.end());
  return v;
}

// The inverse of flat(): the blocks of table t (as mps_table / diag_table give it) filled from v.
inline mps_tensor mps_from_flat(const table& t, uint32_t d, const std::vector<double>& v) {
  mps_tensor A;
  A.d = d;
  A.blocks.resize(d);
  size_t off = 0;
  for (int i = 0; i < t.nblocks(); ++i) {
    key qi(t.qin.begin() + i * t.nsym, t.qin.begin() + (i + 1) * t.nsym);
    key qo(t.qout.begin() + i * t.nsym, t.qout.begin() + (i + 1) * t.nsym);
    dense m;
    m.rows = uint64_t(t.rows[i]);
    m.cols = uint64_t(t.cols[i]);
    if (t.group[i] < 0 || uint32_t(t.group[i]) >= d || off + m.rows * m.cols > v.size())
      throw format_error("table does not match the buffer");
    m.data.assign(v.begin() + off, v.begin() + off + m.rows * m.cols);
    off += m.rows * m.cols;
    A.blocks[t.group[i]][qi] = {qo, std::move(m)};
  }
  return A;
}

inline block_diag diag_from_flat(const table& t, const std::vector<double>& v) {
  block_diag C;
  size_t off = 0;
  for (int i = 0; i < t.nblocks(); ++i) {
    key q(t.qin.begin() + i * t.nsym, t.qin.begin() + (i + 1) * t.nsym);
    dense m;
    m.rows = uint64_t(t.rows[i]);
    m.cols = uint64_t(t.cols[i]);
    if (off + m.rows * m.cols > v.size()) throw format_error("table does not match the buffer");
    m.data.assign(v.begin() + off, v.begin() + off + m.rows * m.cols);
    off += m.rows * m.cols;
    C[q] = std::move(m);
  }
  return C;
}

}  // namespace imps_io
