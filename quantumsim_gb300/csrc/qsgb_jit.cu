// Run-time specialised PTM kernels (NVRTC).
//
// The generic apply kernel (qsgb_apply.cu) interprets per-row term lists from
// shared memory; its loop and indexing overhead costs ~5x the arithmetic of
// a sparse PTM.  When the PTM is on the host, this module instead emits the
// CUDA source of a kernel specialised to the PTM's *sparsity pattern* (which
// entries are non-zero, and for each row whether it is computed in FP64 or
// float-float), compiles it for sm_103a with NVRTC, and caches it by source
// text.  The PTM *values* travel in the kernel parameters, so every PTM with
// the same pattern (e.g. every noisy CZ, whatever its T1/T2) reuses one
// compiled kernel.  The generated kernel keeps the Kin inputs of an item in
// registers, unrolls every row, and issues one load and one store per
// element.
//
// NVRTC is loaded with dlopen on first use; if it is missing or a
// compilation fails, qsgb_jit_apply() returns QSGB_ERR_UNSUPPORTED and the
// caller uses the generic kernel.
#include <dlfcn.h>
#include <nvrtc.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "qsgb_common.cuh"
#include "qsgb_device_src.inc"  // kQsgbDeviceSrc: text of qsgb_device.cuh
#include "qsgb_jit.h"

namespace qsgb {
namespace jit {
namespace {

// ------------------------------------------------------------------ NVRTC
struct Nvrtc {
  bool ok = false;
  nvrtcResult (*create)(nvrtcProgram*, const char*, const char*, int, const char* const*, const char* const*);
  nvrtcResult (*compile)(nvrtcProgram, int, const char* const*);
  nvrtcResult (*log_size)(nvrtcProgram, size_t*);
  nvrtcResult (*log)(nvrtcProgram, char*);
  nvrtcResult (*cubin_size)(nvrtcProgram, size_t*);
  nvrtcResult (*cubin)(nvrtcProgram, char*);
  nvrtcResult (*destroy)(nvrtcProgram*);
};

Nvrtc& nvrtc() {
  static Nvrtc n;
  static std::once_flag once;
  std::call_once(once, [] {
    std::vector<std::string> cands = {"libnvrtc.so.13", "libnvrtc.so"};
    if (const char* h = std::getenv("CUDA_HOME")) cands.push_back(std::string(h) + "/lib64/libnvrtc.so.13");
    cands.push_back("/usr/local/cuda/lib64/libnvrtc.so.13");
    void* lib = nullptr;
    for (const auto& c : cands)
      if ((lib = dlopen(c.c_str(), RTLD_NOW | RTLD_LOCAL))) break;
    if (!lib) return;
    n.create = (decltype(n.create))dlsym(lib, "nvrtcCreateProgram");
    n.compile = (decltype(n.compile))dlsym(lib, "nvrtcCompileProgram");
    n.log_size = (decltype(n.log_size))dlsym(lib, "nvrtcGetProgramLogSize");
    n.log = (decltype(n.log))dlsym(lib, "nvrtcGetProgramLog");
    n.cubin_size = (decltype(n.cubin_size))dlsym(lib, "nvrtcGetCUBINSize");
    n.cubin = (decltype(n.cubin))dlsym(lib, "nvrtcGetCUBIN");
    n.destroy = (decltype(n.destroy))dlsym(lib, "nvrtcDestroyProgram");
    n.ok = n.create && n.compile && n.log_size && n.log && n.cubin_size && n.cubin && n.destroy;
  });
  return n;
}

// Host image of the generated kernel's parameter header (all 8-byte fields,
// so the layout is the same on both sides).
struct Hdr {
  const void* in;
  void* out;
  unsigned* status;
  unsigned long long n_items;
  unsigned long long zm, ym, zd, yd;
  long long zl, yl;
  long long sxi, syi, sai, sbi, sxo, syo, sao, sbo;  // in vector units
};
static_assert(sizeof(Hdr) == 18 * 8, "header layout");
constexpr int kMaxCoef = (32764 - (int)sizeof(Hdr)) / 8;

const char* kHdrSrc =
    "struct H { const void* in; void* out; unsigned* status; qsgb_u64 n_items;\n"
    "  qsgb_u64 zm, ym, zd, yd; qsgb_i64 zl, yl;\n"
    "  qsgb_i64 sxi, syi, sai, sbi, sxo, syo, sao, sbo; };\n";

// ------------------------------------------------------------------ codegen
std::string gen_source(const Spec& s) {
  const int NL = s.pair ? 2 : 1;
  const bool f32 = s.f32;
  const char* scal = f32 ? "float" : "double";
  std::string src;
  src.reserve(16384);
  src += kQsgbDeviceSrc;
  src += "\nstruct __align__(16) qv2d { double x, y; };\nstruct __align__(8) qv2f { float x, y; };\n";
  src += kHdrSrc;
  char buf[4096];
  std::snprintf(buf, sizeof buf, "struct P { H h; double c[%d]; };\n", std::max(1, s.n_coef()));
  src += buf;
  const char* V = s.pair ? (f32 ? "qv2f" : "qv2d") : scal;
  src += "#define QH(v) __int_as_float(__double2hiint(v))\n#define QL(v) __int_as_float(__double2loint(v))\n";
  // vector loads / stores along the less significant target when Z == 1
  {
    const char* ty = f32 ? "f32" : "f64";
    const char* cs = f32 ? "f" : "d";
    std::snprintf(buf, sizeof buf,
                  "__device__ __forceinline__ void qld2(const %s* q, %s& a, %s& b) {\n"
                  "  asm(\"ld.global.nc.v2.%s {%%0,%%1}, [%%2];\" : \"=%s\"(a), \"=%s\"(b) : \"l\"(q)); }\n"
                  "__device__ __forceinline__ void qld4(const %s* q, %s& a, %s& b, %s& c, %s& d) {\n"
                  "  asm(\"ld.global.nc.v4.%s {%%0,%%1,%%2,%%3}, [%%4];\" : \"=%s\"(a), \"=%s\"(b), \"=%s\"(c), "
                  "\"=%s\"(d) : \"l\"(q)); }\n"
                  "__device__ __forceinline__ void qst2(%s* q, %s a, %s b) {\n"
                  "  asm volatile(\"st.global.v2.%s [%%0], {%%1,%%2};\" :: \"l\"(q), \"%s\"(a), \"%s\"(b) : \"memory\"); }\n"
                  "__device__ __forceinline__ void qst4(%s* q, %s a, %s b, %s c, %s d) {\n"
                  "  asm volatile(\"st.global.v4.%s [%%0], {%%1,%%2,%%3,%%4};\" :: \"l\"(q), \"%s\"(a), \"%s\"(b), "
                  "\"%s\"(c), \"%s\"(d) : \"memory\"); }\n",
                  scal, scal, scal, ty, cs, cs, scal, scal, scal, scal, scal, ty, cs, cs, cs, cs, scal, scal, scal, ty, cs,
                  cs, scal, scal, scal, scal, scal, ty, cs, cs, cs, cs);
    src += buf;
  }
  std::snprintf(buf, sizeof buf,
                "extern \"C\" __global__ void __launch_bounds__(128) qsgb_jit(const __grid_constant__ P p) {\n"
                "  typedef %s V;\n"
                "  const V* __restrict__ in = (const V*)p.h.in;\n"
                "  V* __restrict__ out = (V*)p.h.out;\n"
                "  unsigned bad = 0;\n"
                "  const qsgb_u64 stride = (qsgb_u64)gridDim.x * blockDim.x;\n"
                "  for (qsgb_u64 it = (qsgb_u64)blockIdx.x * blockDim.x + threadIdx.x; it < p.h.n_items; it += "
                "stride) {\n"
                "    const qsgb_u64 t1 = qsgb_fdiv(it, p.h.zm, (int)p.h.zl);\n"
                "    const qsgb_u64 zi = it - t1 * p.h.zd;\n"
                "    const qsgb_u64 xx = qsgb_fdiv(t1, p.h.ym, (int)p.h.yl);\n"
                "    const qsgb_u64 yy = t1 - xx * p.h.yd;\n"
                "    const qsgb_i64 bi = (qsgb_i64)xx * p.h.sxi + (qsgb_i64)yy * p.h.syi + (qsgb_i64)zi;\n"
                "    const qsgb_i64 bo = (qsgb_i64)xx * p.h.sxo + (qsgb_i64)yy * p.h.syo + (qsgb_i64)zi;\n",
                V);
  src += buf;
  // which inputs are used, and which feed df rows
  std::vector<char> used(s.kin, 0), split(s.kin, 0);
  for (int r = 0; r < s.kout; ++r)
    for (int k : s.cols[r]) {
      used[k] = 1;
      if (s.mode[r] == kModeDF) split[k] = 1;
    }
  const char* lanes[2] = {s.pair ? ".x" : "", ".y"};
  if (s.vin > 1) {  // Z == 1: runs of vin inputs along kb are contiguous
    for (int k0 = 0; k0 < s.kin; k0 += s.vin) {
      bool any = false;
      for (int j = 0; j < s.vin; ++j) any |= used[k0 + j] != 0;
      if (!any) continue;
      const int ka = k0 / s.db_in, kb = k0 % s.db_in;
      std::string vars;
      for (int j = 0; j < s.vin; ++j) {
        std::snprintf(buf, sizeof buf, "    V x%d;\n", k0 + j);
        src += buf;
        vars += ", x" + std::to_string(k0 + j);
      }
      std::snprintf(buf, sizeof buf, "    qld%d((const V*)p.h.in + bi + %dLL * p.h.sai + %d%s);\n", s.vin, ka, kb,
                    vars.c_str());
      src += buf;
    }
  } else {
    for (int k = 0; k < s.kin; ++k) {
      if (!used[k]) continue;
      const int ka = k / s.db_in, kb = k % s.db_in;
      std::snprintf(buf, sizeof buf, "    const V x%d = in[bi + %dLL * p.h.sai + %dLL * p.h.sbi];\n", k, ka, kb);
      src += buf;
    }
  }
  for (int k = 0; k < s.kin; ++k) {
    if (!split[k]) continue;
    for (int l = 0; l < NL; ++l) {
      std::snprintf(buf, sizeof buf, "    float h%d_%d, l%d_%d; qsgb_split_f64(x%d%s, h%d_%d, l%d_%d, bad);\n", k, l, k,
                    l, k, lanes[l], k, l, k, l);
      src += buf;
    }
  }
  for (int r = 0; r < s.kout; ++r) {
    std::snprintf(buf, sizeof buf, "    V y%d;\n", r);
    src += buf;
  }
  int ci = 0;
  for (int r = 0; r < s.kout; ++r) {
    const int ra = r / s.db_out, rb = r % s.db_out;
    const auto& cols = s.cols[r];
    src += "    {\n";
    std::string vals[2];
    for (int l = 0; l < NL; ++l) {
      if (cols.empty()) {
        vals[l] = f32 ? "0.f" : "0.0";
        continue;
      }
      if (f32) {
        std::snprintf(buf, sizeof buf, "      float a%d = QL(p.c[%d]) * x%d%s;\n", l, ci, cols[0], lanes[l]);
        src += buf;
        for (size_t j = 1; j < cols.size(); ++j) {
          std::snprintf(buf, sizeof buf, "      a%d = fmaf(QL(p.c[%d]), x%d%s, a%d);\n", l, ci + (int)j, cols[j],
                        lanes[l], l);
          src += buf;
        }
        vals[l] = "a" + std::to_string(l);
      } else if (s.mode[r] == kModeDP) {
        std::snprintf(buf, sizeof buf, "      double a%d = p.c[%d] * x%d%s;\n", l, ci, cols[0], lanes[l]);
        src += buf;
        for (size_t j = 1; j < cols.size(); ++j) {
          std::snprintf(buf, sizeof buf, "      a%d = fma(p.c[%d], x%d%s, a%d);\n", l, ci + (int)j, cols[j], lanes[l],
                        l);
          src += buf;
        }
        vals[l] = "a" + std::to_string(l);
      } else {
        std::snprintf(buf, sizeof buf,
                      "      float s%d, c%d; qsgb_df_mul(s%d, c%d, QH(p.c[%d]), QL(p.c[%d]), h%d_%d, l%d_%d);\n", l, l,
                      l, l, ci, ci, cols[0], l, cols[0], l);
        src += buf;
        for (size_t j = 1; j < cols.size(); ++j) {
          const int q = ci + (int)j;
          std::snprintf(buf, sizeof buf, "      qsgb_df_fma(s%d, c%d, QH(p.c[%d]), QL(p.c[%d]), h%d_%d, l%d_%d);\n", l,
                        l, q, q, cols[j], l, cols[j], l);
          src += buf;
        }
        vals[l] = "qsgb_df_to_double(s" + std::to_string(l) + ", c" + std::to_string(l) + ")";
      }
    }
    if (s.pair) {
      src += "      y" + std::to_string(r) + ".x = " + vals[0] + "; y" + std::to_string(r) + ".y = " + vals[1] + ";\n";
    } else {
      src += "      y" + std::to_string(r) + " = " + vals[0] + ";\n";
    }
    src += "    }\n";
    ci += (int)cols.size();
    // store as soon as a row (or a vector of vout rows) is complete
    if (s.vout > 1) {
      if ((r + 1) % s.vout == 0) {
        const int r0 = r + 1 - s.vout;
        std::string vars;
        for (int j = 0; j < s.vout; ++j) vars += ", y" + std::to_string(r0 + j);
        std::snprintf(buf, sizeof buf, "    qst%d((V*)p.h.out + bo + %dLL * p.h.sao + %d%s);\n", s.vout,
                      r0 / s.db_out, r0 % s.db_out, vars.c_str());
        src += buf;
      }
    } else {
      std::snprintf(buf, sizeof buf, "    out[bo + %dLL * p.h.sao + %dLL * p.h.sbo] = y%d;\n", ra, rb, r);
      src += buf;
    }
  }
  src += "  }\n  if (bad && p.h.status) atomicOr(p.h.status, 1u);\n}\n";
  return src;
}

struct Cache {
  std::mutex mu;
  std::unordered_map<std::string, cudaKernel_t> kernels;
  std::unordered_map<std::string, int> failed;
};
Cache& cache() {
  static Cache c;
  return c;
}

// On-disk cubin cache: $QSGB_JIT_CACHE, default <package>/_build/jit_cache
// (next to libqsgb.so), file name = FNV-1a hash of the source + its length.
std::string cache_path(const std::string& src) {
  std::string dir;
  if (const char* d = std::getenv("QSGB_JIT_CACHE")) {
    dir = d;
  } else {
    Dl_info info;
    if (!dladdr((void*)&cache_path, &info) || !info.dli_fname) return "";
    dir = info.dli_fname;
    const size_t slash = dir.rfind('/');
    dir = (slash == std::string::npos ? std::string(".") : dir.substr(0, slash)) + "/_build/jit_cache";
  }
  unsigned long long h = 1469598103934665603ull;
  for (unsigned char ch : src) h = (h ^ ch) * 1099511628211ull;
  char name[64];
  std::snprintf(name, sizeof name, "/%016llx_%zu.cubin", h, src.size());
  return dir + name;
}

bool read_file(const std::string& path, std::vector<char>& data) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  const long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  data.resize(n > 0 ? (size_t)n : 0);
  const bool ok = n > 0 && std::fread(data.data(), 1, data.size(), f) == data.size();
  std::fclose(f);
  return ok;
}

void write_file(const std::string& path, const std::vector<char>& data) {
  const size_t slash = path.rfind('/');
  if (slash != std::string::npos) {
    // create the directory (and its parent) if needed
    const std::string dir = path.substr(0, slash);
    const size_t up = dir.rfind('/');
    if (up != std::string::npos) mkdir(dir.substr(0, up).c_str(), 0755);
    mkdir(dir.c_str(), 0755);
  }
  const std::string tmp = path + ".tmp" + std::to_string((unsigned long)getpid());
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) return;
  const bool ok = std::fwrite(data.data(), 1, data.size(), f) == data.size();
  std::fclose(f);
  if (ok) std::rename(tmp.c_str(), path.c_str()); else std::remove(tmp.c_str());
}

int load_cubin(const std::vector<char>& cubin, cudaKernel_t* out) {
  cudaLibrary_t lib;
  if (cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0) != cudaSuccess) {
    cudaGetLastError();
    return QSGB_ERR_CUDA;
  }
  if (cudaLibraryGetKernel(out, lib, "qsgb_jit") != cudaSuccess) {
    cudaGetLastError();
    return QSGB_ERR_CUDA;
  }
  return QSGB_OK;
}

int compile(const std::string& src, cudaKernel_t* out) {
  const std::string path = cache_path(src);
  std::vector<char> cubin;
  if (!path.empty() && read_file(path, cubin) && load_cubin(cubin, out) == QSGB_OK) return QSGB_OK;
  Nvrtc& n = nvrtc();
  if (!n.ok) return QSGB_ERR_UNSUPPORTED;
  nvrtcProgram prog;
  if (n.create(&prog, src.c_str(), "qsgb_jit.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) return QSGB_ERR_UNSUPPORTED;
  const char* opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "-default-device"};
  const nvrtcResult cr = n.compile(prog, 3, opts);
  if (cr != NVRTC_SUCCESS) {
    if (std::getenv("QSGB_JIT_VERBOSE")) {
      size_t ls = 0;
      n.log_size(prog, &ls);
      std::string log(ls, '\0');
      n.log(prog, &log[0]);
      std::fprintf(stderr, "qsgb jit: compilation failed:\n%s\n", log.c_str());
    }
    n.destroy(&prog);
    return QSGB_ERR_UNSUPPORTED;
  }
  size_t sz = 0;
  n.cubin_size(prog, &sz);
  cubin.assign(sz, 0);
  n.cubin(prog, cubin.data());
  n.destroy(&prog);
  const int st = load_cubin(cubin, out);
  if (st == QSGB_OK && !path.empty()) write_file(path, cubin);
  return st;
}

}  // namespace

int Spec::n_coef() const {
  int n = 0;
  for (const auto& c : cols) n += (int)c.size();
  return n;
}

bool available() { return nvrtc().ok && !std::getenv("QSGB_NO_JIT"); }

int kernel_for(const Spec& s, cudaKernel_t* k, std::string* src_out) {
  if (s.n_coef() > kMaxCoef) return QSGB_ERR_UNSUPPORTED;
  const std::string src = gen_source(s);
  if (src_out) *src_out = src;
  Cache& c = cache();
  {
    std::lock_guard<std::mutex> g(c.mu);
    auto it = c.kernels.find(src);
    if (it != c.kernels.end()) {
      *k = it->second;
      return QSGB_OK;
    }
    if (c.failed.count(src)) return QSGB_ERR_UNSUPPORTED;
  }
  cudaKernel_t kern;
  const int st = compile(src, &kern);
  std::lock_guard<std::mutex> g(c.mu);
  if (st != QSGB_OK) {
    c.failed[src] = st;
    return QSGB_ERR_UNSUPPORTED;
  }
  c.kernels[src] = kern;
  *k = kern;
  return QSGB_OK;
}

int launch(const Spec& s, const Geometry& g, const double* coef, cudaStream_t stream) {
  cudaKernel_t kern;
  const int st = kernel_for(s, &kern, nullptr);
  if (st != QSGB_OK) return st;
  const int nc = std::max(1, s.n_coef());
  std::vector<unsigned char> blob(sizeof(Hdr) + 8 * (size_t)nc, 0);
  Hdr h;
  h.in = g.in;
  h.out = g.out;
  h.status = g.status;
  h.n_items = g.n_items;
  h.zm = g.div_z.m;
  h.zd = g.div_z.d;
  h.zl = g.div_z.l;
  h.ym = g.div_y.m;
  h.yd = g.div_y.d;
  h.yl = g.div_y.l;
  h.sxi = g.sxi;
  h.syi = g.syi;
  h.sai = g.sai;
  h.sbi = g.sbi;
  h.sxo = g.sxo;
  h.syo = g.syo;
  h.sao = g.sao;
  h.sbo = g.sbo;
  std::memcpy(blob.data(), &h, sizeof h);
  std::memcpy(blob.data() + sizeof h, coef, 8 * (size_t)s.n_coef());
  void* args[] = {blob.data()};
  const unsigned block = 128;
  const uint64_t need = (g.n_items + block - 1) / block;
  const uint64_t cap = (uint64_t)sm_count() * 16;
  const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min(need, cap));
  QSGB_CUDA_TRY(cudaLaunchKernel((const void*)kern, dim3(grid), dim3(block), args, 0, stream));
  return QSGB_OK;
}

}  // namespace jit
}  // namespace qsgb

extern "C" int qsgb_jit_available(void) { return qsgb::jit::available() ? 1 : 0; }
