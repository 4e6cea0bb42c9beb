// Binary model cache: the packed (device-layout) model in one little-endian file, so
// that a large libsymmetrix JSON (hundreds of MB at 128 channels, seconds to parse;
// MACE::load_from_json, libsymmetrix/source/mace.cpp:905-1030) is parsed once.
//
// Layout: magic "SMXGB300", format version, then every field of PackedModel and the
// HostModel scalars the engine reads, in declaration order; vectors as (uint64 count,
// elements).  A cache file is a standalone model: smx_create accepts it in place of
// the JSON (recognised by the magic).
#include <cstdint>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "model.hpp"

namespace smx {

namespace {

constexpr char kMagic[8] = {'S', 'M', 'X', 'G', 'B', '3', '0', '0'};
constexpr uint32_t kVersion = 2;

struct Out {
  std::ofstream f;
  template <typename T>
  void put(const T& v) {
    static_assert(std::is_trivially_copyable<T>::value, "plain data only");
    f.write(reinterpret_cast<const char*>(&v), sizeof(T));
  }
  template <typename T>
  void vec(const std::vector<T>& v) {
    put(static_cast<uint64_t>(v.size()));
    if (!v.empty()) f.write(reinterpret_cast<const char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(T)));
  }
};

struct In {
  std::ifstream f;
  template <typename T>
  void get(T& v) {
    f.read(reinterpret_cast<char*>(&v), sizeof(T));
    if (!f) throw std::invalid_argument("model cache: truncated file");
  }
  template <typename T>
  void vec(std::vector<T>& v) {
    uint64_t n = 0;
    get(n);
    if (n > (uint64_t(1) << 36)) throw std::invalid_argument("model cache: corrupt vector length");
    v.resize(n);
    if (n) f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(n * sizeof(T)));
    if (!f) throw std::invalid_argument("model cache: truncated file");
  }
};

}  // namespace

bool is_model_cache(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  char m[8] = {};
  f.read(m, 8);
  return f && std::memcmp(m, kMagic, 8) == 0;
}

#define SMX_CACHE_FIELDS(X, V)                                                                              \
  X(hm.S) X(hm.C) X(hm.l_max) X(hm.L_max) X(hm.nLM) X(hm.r_cut) V(hm.Z) X(hm.spl_h) X(hm.has_zbl)           \
  X(hm.A0_scaled) X(hm.A1_scaled)                                                                           \
  X(pm.S) X(pm.C) X(pm.L_max) X(pm.nLM) X(pm.n_lme) X(pm.n_instr) X(pm.n_p) X(pm.nint) X(pm.npairs) X(pm.h) \
  X(pm.r_cut) V(pm.spl0) V(pm.spl1) V(pm.spl1_fwd) V(pm.mono0) V(pm.mono0_off) X(pm.T0) V(pm.coef0)          \
  V(pm.mono1) X(pm.T1) V(pm.coef1) X(pm.poly_canon) V(pm.H1W) V(pm.H1W_T) V(pm.cg_fwd_off) V(pm.cg_fwd_p)    \
  V(pm.cg_fwd_v) V(pm.cg_rev_off) V(pm.cg_rev_lme) V(pm.cg_rev_v) X(pm.lme_off) X(pm.num_e) V(pm.A1W[0])      \
  V(pm.A1W[1]) V(pm.A1W[2]) V(pm.A1W[3]) V(pm.A1W_T[0]) V(pm.A1W_T[1]) V(pm.A1W_T[2]) V(pm.A1W_T[3])         \
  V(pm.H2W_H1) V(pm.H2W_H1_T) V(pm.H2W_M1) V(pm.H2W_M1_T) V(pm.ro1) V(pm.ro2_w1) V(pm.ro2_w2)                \
  X(pm.ro2_scale) X(pm.n_hidden) V(pm.e0) V(pm.Z) X(pm.has_zbl) X(pm.zbl_p) X(pm.zbl_c) V(pm.zbl_pair) \
  X(pm.dens_scaled) X(pm.dens_nint) X(pm.dens_h) V(pm.dens_spl[0]) V(pm.dens_spl[1])

void save_model_cache(const std::string& path, const HostModel& hm, const PackedModel& pm) {
  Out o;
  o.f.open(path, std::ios::binary | std::ios::trunc);
  if (!o.f) throw std::invalid_argument("model cache: cannot write " + path);
  o.f.write(kMagic, 8);
  o.put(kVersion);
#define SMX_X(v) o.put(v);
#define SMX_V(v) o.vec(v);
  SMX_CACHE_FIELDS(SMX_X, SMX_V)
#undef SMX_X
#undef SMX_V
  if (!o.f) throw std::invalid_argument("model cache: write failed for " + path);
}

void load_model_cache(const std::string& path, HostModel& hm, PackedModel& pm) {
  In in;
  in.f.open(path, std::ios::binary);
  if (!in.f) throw std::invalid_argument("model cache: cannot open " + path);
  char m[8];
  in.f.read(m, 8);
  uint32_t ver = 0;
  in.get(ver);
  if (std::memcmp(m, kMagic, 8) != 0 || ver != kVersion)
    throw std::invalid_argument("model cache: not a cache file of this format version");
#define SMX_X(v) in.get(v);
#define SMX_V(v) in.vec(v);
  SMX_CACHE_FIELDS(SMX_X, SMX_V)
#undef SMX_X
#undef SMX_V
}

}  // namespace smx
