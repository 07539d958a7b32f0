// Run-time specialised PTM kernels (NVRTC).
//
// The generic apply kernel (qsgb_apply.cu) interprets per-row term lists from
// shared memory; its loop and indexing overhead costs ~5x the arithmetic of
// a sparse PTM.  When the PTM is on the host, this module instead emits the
// CUDA source of a kernel specialised to the PTM's *sparsity pattern* (which
// entries are non-zero, and for each row whether it is computed in FP64 or
// float-float), compiles it for sm_103a with NVRTC, and caches it (in
// process by pattern, on disk by source text).  The PTM *values* travel in
// the kernel parameters, so every PTM with the same pattern (e.g. every
// noisy CZ, whatever its T1/T2) reuses one compiled kernel.  The generated
// kernel holds an item's inputs in registers, unrolls every row, and issues
// one load and one store per element.
//
// NVRTC is loaded with dlopen on first use; if it is missing or a
// compilation fails, launch() returns QSGB_ERR_UNSUPPORTED and the caller
// uses the generic kernel.
#include <dlfcn.h>
#include <nvrtc.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
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
// Patterns with more terms are left to the generic kernel: they are
// arithmetic-bound whatever the code, and NVRTC needs 12-65 s for a 2000-term
// 81x81 pattern (255 registers plus spills), against ~1 s for the sparse
// PTMs of physical gates (<= 256 terms).
constexpr int kMaxJitTerms = 1024;

const char* kHdrSrc =
    "struct H { const void* in; void* out; unsigned* status; qsgb_u64 n_items;\n"
    "  qsgb_u64 zm, ym, zd, yd; qsgb_i64 zl, yl;\n"
    "  qsgb_i64 sxi, syi, sai, sbi, sxo, syo, sao, sbo; };\n";

// ------------------------------------------------------------------ codegen
// Component id (its smallest row) of every row of the row/column graph: two
// rows are connected when they read a common input.
std::vector<int> row_components(const Spec& s) {
  std::vector<int> parent(s.kout);
  for (int r = 0; r < s.kout; ++r) parent[r] = r;
  auto find = [&](int r) {
    while (parent[r] != r) r = parent[r] = parent[parent[r]];
    return r;
  };
  std::vector<int> first_row(s.kin, -1);
  for (int r = 0; r < s.kout; ++r)
    for (int k : s.cols[r]) {
      if (first_row[k] < 0) {
        first_row[k] = r;
      } else {
        const int a = find(first_row[k]), b = find(r);
        if (a != b) parent[std::max(a, b)] = std::min(a, b);
      }
    }
  std::vector<int> comp(s.kout);
  for (int r = 0; r < s.kout; ++r) comp[r] = find(r);
  return comp;
}

// Rows grouped by component, components in order of their first row, rows
// ascending within a component.
std::vector<int> row_order(const Spec& s) {
  const std::vector<int> comp = row_components(s);
  std::vector<std::vector<int>> members(s.kout);
  for (int r = 0; r < s.kout; ++r) members[comp[r]].push_back(r);
  std::vector<int> order;
  order.reserve(s.kout);
  for (int r = 0; r < s.kout; ++r)
    for (int m : members[r]) order.push_back(m);
  return order;
}

// A staged kernel writes each component's results over the tile slots of
// their own row indices; that is safe when no later component reads those
// slots as inputs.
bool staged_in_place_ok(const Spec& s) {
  if (s.lookahead >= s.kin) return true;  // all inputs are read before any write
  const std::vector<int> order = row_order(s);
  const std::vector<int> comp = row_components(s);
  std::vector<int> at(s.kout);
  for (size_t i = 0; i < order.size(); ++i) at[order[i]] = (int)i;
  // position of the last row of each component, and of the last reader of each input
  std::vector<int> comp_end(s.kout, -1), last_read(s.kin, -1);
  for (int r = 0; r < s.kout; ++r) {
    comp_end[comp[r]] = std::max(comp_end[comp[r]], at[r]);
    for (int k : s.cols[r]) last_read[k] = std::max(last_read[k], at[r]);
  }
  for (int r = 0; r < s.kout && r < s.kin; ++r)
    if (last_read[r] > comp_end[comp[r]]) return false;
  return true;
}

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
  // Float-float rows of an item whose inputs or results leave the range of
  // the float pair (qsgb_split_f64, qsgb_df_suspect) are computed again in
  // native FP64 from the input, which the kernel does not overwrite (it
  // writes a separate output): a loop over tables of the pattern's terms,
  // kept out of the unrolled hot path.
  std::string fallback;
  if (std::count(s.mode.begin(), s.mode.end(), (int)kModeDF) > 0) {
    std::string tk, te, td;
    int t = 0;
    for (int r = 0; r < s.kout; ++r) {
      for (int k : s.cols[r]) tk += std::to_string(k) + ",";
      t += (int)s.cols[r].size();
      te += std::to_string(t) + ",";
      td += s.mode[r] == kModeDF ? "1," : "0,";
    }
    if (tk.empty()) tk = "0,";
    src += "__constant__ unsigned short qfb_k[] = {" + tk + "};\n";
    src += "__constant__ unsigned short qfb_end[] = {" + te + "};\n";
    src += "__constant__ unsigned char qfb_df[] = {" + td + "};\n";
    const bool staged = s.stage_warps > 0;
    std::snprintf(buf, sizeof buf,
                  "    if (fb%s) {\n"
                  "      unsigned tq = 0;\n"
                  "#pragma unroll 1\n"
                  "      for (int r = 0; r < %d; ++r) {\n"
                  "        const unsigned te = qfb_end[r];\n"
                  "        if (!qfb_df[r]) { tq = te; continue; }\n"
                  "        double a0 = 0.0, a1 = 0.0;\n"
                  "#pragma unroll 1\n"
                  "        for (; tq < te; ++tq) {\n"
                  "          const unsigned k = qfb_k[tq];\n"
                  "          const double cf = (double)QH(p.c[tq]) + (double)QL(p.c[tq]);\n"
                  "          const V xv = in[bi + (qsgb_i64)(k / %du) * p.h.sai + (qsgb_i64)(k %% %du) * %s];\n"
                  "%s"
                  "        }\n"
                  "%s"
                  "      }\n"
                  "    }\n",
                  staged ? " && lane < nv" : "", s.kout, s.db_in, s.db_in, staged ? "1" : "p.h.sbi",
                  s.pair ? "          a0 = fma(cf, xv.x, a0); a1 = fma(cf, xv.y, a1);\n"
                         : "          a0 = fma(cf, xv, a0);\n",
                  "");
    fallback = buf;
    // where the row's result goes
    std::string store;
    if (staged) {
      std::snprintf(buf, sizeof buf, "        t[lane * %d + r] = a0; (void)a1;\n", std::max(s.kin, s.kout));
      store = buf;
    } else {
      std::snprintf(buf, sizeof buf,
                    "        { V yv; %s out[bo + (qsgb_i64)(r / %d) * p.h.sao + (qsgb_i64)(r %% %d) * p.h.sbo] = yv; }\n",
                    s.pair ? "yv.x = a0; yv.y = a1;" : "yv = a0; (void)a1;", s.db_out, s.db_out);
      store = buf;
    }
    const size_t at = fallback.rfind("      }\n    }\n");
    fallback.insert(at, store);
  }
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
  const int KS = std::max(s.kin, s.kout);  // staged tile: values per item
  if (s.stage_warps) {
    // Z == 1 with odd (or unaligned) target dims: each warp stages the items
    // of 32 consecutive groups in shared memory with coalesced copies,
    // computes from there, and writes the results back through the same
    // tile.  When the 32 groups form one contiguous span (stage_bulk: one
    // qudit, or two adjacent last qudits; square PTM), one bulk copy (TMA,
    // completion on an mbarrier) moves the tile each way; a tile whose size
    // is not a multiple of 16 bytes uses the per-element copies.
    const int esz = f32 ? 4 : 8;
    std::snprintf(buf, sizeof buf,
                  "extern \"C\" __global__ void __launch_bounds__(%d) qsgb_jit(const __grid_constant__ P p) {\n"
                  "  typedef %s V;\n"
                  "  __shared__ __align__(128) V tiles[%d][32 * %d];\n"
                  "  V* const t = tiles[threadIdx.x >> 5];\n"
                  "  const unsigned lane = threadIdx.x & 31u;\n"
                  "  const V* __restrict__ in = (const V*)p.h.in;\n"
                  "  V* __restrict__ out = (V*)p.h.out;\n"
                  "  const unsigned tb = (unsigned)__cvta_generic_to_shared(t);\n"
                  "",
                  32 * s.stage_warps, scal, s.stage_warps, KS);
    src += buf;
    if (s.stage_bulk) {
      std::snprintf(buf, sizeof buf,
                    "  __shared__ __align__(8) qsgb_u64 bars[%d];\n"
                    "  const unsigned bar = (unsigned)__cvta_generic_to_shared(&bars[threadIdx.x >> 5]);\n"
                    "  if (lane == 0) {\n"
                    "    asm volatile(\"mbarrier.init.shared::cta.b64 [%%0], 1;\" :: \"r\"(bar) : \"memory\");\n"
                    "    asm volatile(\"fence.proxy.async.shared::cta;\" ::: \"memory\");\n"
                    "  }\n"
                    "  __syncwarp();\n"
                    "  unsigned phase = 0;\n",
                    s.stage_warps);
      src += buf;
    }
    std::snprintf(buf, sizeof buf,
                  "  const qsgb_u64 n_tiles = (p.h.n_items + 31) >> 5;\n"
                  "  const qsgb_u64 wstride = (qsgb_u64)gridDim.x * %d;\n"
                  "  for (qsgb_u64 wt = (qsgb_u64)blockIdx.x * %d + (threadIdx.x >> 5); wt < n_tiles; wt += wstride) "
                  "{\n"
                  "    const qsgb_u64 left = p.h.n_items - wt * 32;\n"
                  "    const unsigned nv = left < 32 ? (unsigned)left : 32u;\n"
                  "    qsgb_i64 bi = 0, bo = 0;\n"
                  "    if (lane < nv) {\n"
                  "      const qsgb_u64 it = wt * 32 + lane;\n"
                  "      const qsgb_u64 xx = qsgb_fdiv(it, p.h.ym, (int)p.h.yl);\n"
                  "      const qsgb_u64 yy = it - xx * p.h.yd;\n"
                  "      bi = (qsgb_i64)xx * p.h.sxi + (qsgb_i64)yy * p.h.syi;\n"
                  "      bo = (qsgb_i64)xx * p.h.sxo + (qsgb_i64)yy * p.h.syo;\n"
                  "    }\n"
                  "    unsigned fb = 0;  // the item needs native FP64 (input or result range)\n",
                  s.stage_warps, s.stage_warps);
    src += buf;
    if (s.stage_bulk) {
      std::snprintf(buf, sizeof buf,
                    "    const unsigned nbytes = nv * %du;\n"
                    "    const bool bulk = (nbytes & 15u) == 0u;\n"
                    "    if (bulk) {\n"
                    "      if (lane == 0) {\n"
                    "        // the previous tile's store has finished reading the tile\n"
                    "        asm volatile(\"cp.async.bulk.wait_group.read 0;\" ::: \"memory\");\n"
                    "        asm volatile(\"mbarrier.arrive.expect_tx.shared::cta.b64 _, [%%0], %%1;\" :: \"r\"(bar), "
                    "\"r\"(nbytes) : \"memory\");\n"
                    "        asm volatile(\"cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%%0], "
                    "[%%1], %%2, [%%3];\" :: \"r\"(tb), \"l\"(in + wt * %du), \"r\"(nbytes), \"r\"(bar) : \"memory\");\n"
                    "      }\n"
                    "      // bounded wait for the tile (parity of this warp's barrier phase)\n"
                    "      unsigned ok = 0;\n"
                    "      for (unsigned spin = 0; spin < (1u << 24) && !ok; ++spin) {\n"
                    "        unsigned w;\n"
                    "        asm volatile(\"{ .reg .pred q; mbarrier.try_wait.parity.shared::cta.b64 q, [%%1], %%2; "
                    "selp.u32 %%0, 1, 0, q; }\" : \"=r\"(w) : \"r\"(bar), \"r\"(phase) : \"memory\");\n"
                    "        ok = __all_sync(0xffffffffu, w != 0u);\n"
                    "      }\n"
                    "      phase ^= 1u;\n"
                    "      if (!ok) {\n"
                    "        if (lane == 0 && p.h.status) atomicOr(p.h.status, 2u);\n"
                    "        break;\n"
                    "      }\n"
                    "    } else {\n"
                    "      if (lane == 0) asm volatile(\"cp.async.bulk.wait_group.read 0;\" ::: \"memory\");\n"
                    "      __syncwarp();\n",
                    KS * esz, 32 * KS);
      src += buf;
    }
    // lane copies elements f = lane + 32 j of each run of db values (one run
    // per item and ka): item i = f / db, offset kb = f % db, with the item's
    // base taken from lane i
    std::snprintf(buf, sizeof buf,
                  "    // coalesced global -> shared copies (cp.async: no registers held)\n"
                  "    qsgb_i64 srcj[%d];\n"
                  "#pragma unroll\n"
                  "    for (int j = 0; j < %d; ++j) srcj[j] = __shfl_sync(0xffffffffu, bi, (lane + 32u * j) / %du);\n"
                  "#pragma unroll 3\n"
                  "    for (int ka = 0; ka < %d; ++ka) {\n"
                  "#pragma unroll\n"
                  "      for (int j = 0; j < %d; ++j) {\n"
                  "        const unsigned f = lane + 32u * j, i = f / %du, kb = f - i * %du;\n"
                  "        if (i < nv)\n"
                  "          asm volatile(\"cp.async.ca.shared.global [%%0], [%%1], %d;\" :: \"r\"(tb + (i * %du + ka * "
                  "%du + kb) * %du), \"l\"(in + srcj[j] + ka * p.h.sai + kb) : \"memory\");\n"
                  "      }\n"
                  "    }\n"
                  "    asm volatile(\"cp.async.wait_all;\" ::: \"memory\");\n"
                  "%s"
                  "    __syncwarp();\n",
                  s.db_in, s.db_in, s.db_in, s.kin / s.db_in, s.db_in, s.db_in, s.db_in, esz, KS, s.db_in, esz,
                  s.stage_bulk ? "    }\n" : "");
    src += buf;
  } else {
  std::snprintf(buf, sizeof buf,
                "extern \"C\" __global__ void __launch_bounds__(128) qsgb_jit(const __grid_constant__ P p) {\n"
                "  typedef %s V;\n"
                "  const V* __restrict__ in = (const V*)p.h.in;\n"
                "  V* __restrict__ out = (V*)p.h.out;\n"
                "  const qsgb_u64 stride = (qsgb_u64)gridDim.x * blockDim.x;\n"
                "  for (qsgb_u64 it = (qsgb_u64)blockIdx.x * blockDim.x + threadIdx.x; it < p.h.n_items; it += "
                "stride) {\n"
                "    const qsgb_u64 t1 = qsgb_fdiv(it, p.h.zm, (int)p.h.zl);\n"
                "    const qsgb_u64 zi = it - t1 * p.h.zd;\n"
                "    const qsgb_u64 xx = qsgb_fdiv(t1, p.h.ym, (int)p.h.yl);\n"
                "    const qsgb_u64 yy = t1 - xx * p.h.yd;\n"
                "    const qsgb_i64 bi = (qsgb_i64)xx * p.h.sxi + (qsgb_i64)yy * p.h.syi + (qsgb_i64)zi;\n"
                "    const qsgb_i64 bo = (qsgb_i64)xx * p.h.sxo + (qsgb_i64)yy * p.h.syo + (qsgb_i64)zi;\n"
                "    unsigned fb = 0;  // the item needs native FP64 (input or result range)\n",
                V);
  src += buf;
  }
  const char* lanes[2] = {s.pair ? ".x" : "", ".y"};
  // Small items load (and split) every input first and emit rows in natural
  // order.  Large ones emit rows component by component (rows that share an
  // input form one component of the row/column graph), each input loaded a
  // few inputs ahead of its first use, so the live registers of an item are
  // those of a few components rather than all Kin inputs.  Every result is
  // stored as soon as it (or its vector of vout results) is complete.
  std::vector<int> order(s.kout);
  if (s.lookahead >= s.kin) {
    for (int r = 0; r < s.kout; ++r) order[r] = r;
  } else {
    order = row_order(s);
  }
  // comp_last[r]: r is the last row (in `order`) of its component; with all
  // inputs loaded first the whole row set counts as one component
  std::vector<char> comp_last(s.kout, 0);
  {
    const std::vector<int> comp = row_components(s);
    for (size_t i = 0; i < order.size(); ++i) {
      const bool last = i + 1 == order.size() ||
                        (s.lookahead < s.kin && comp[order[i + 1]] != comp[order[i]]);
      comp_last[order[i]] = last ? 1 : 0;
    }
  }
  std::vector<int> pending;
  std::vector<int> ci0(s.kout + 1, 0);
  for (int r = 0; r < s.kout; ++r) ci0[r + 1] = ci0[r] + (int)s.cols[r].size();
  std::vector<char> loaded(s.kin, 0), splitd(s.kin, 0), done(s.kout, 0);
  auto load = [&](int k) {
    if (s.vin > 1) {  // Z == 1: runs of vin inputs along kb are contiguous
      const int k0 = k - k % s.vin;
      if (loaded[k0]) return;
      std::string vars;
      for (int j = 0; j < s.vin; ++j) {
        loaded[k0 + j] = 1;
        std::snprintf(buf, sizeof buf, "    V x%d;\n", k0 + j);
        src += buf;
        vars += ", x" + std::to_string(k0 + j);
      }
      std::snprintf(buf, sizeof buf, "    qld%d((const V*)p.h.in + bi + %dLL * p.h.sai + %d%s);\n", s.vin,
                    k0 / s.db_in, k0 % s.db_in, vars.c_str());
      src += buf;
    } else {
      if (loaded[k]) return;
      loaded[k] = 1;
      if (s.stage_warps)
        std::snprintf(buf, sizeof buf, "    const V x%d = t[lane * %d + %d];\n", k, KS, k);
      else
        std::snprintf(buf, sizeof buf, "    const V x%d = in[bi + %dLL * p.h.sai + %dLL * p.h.sbi];\n", k,
                      k / s.db_in, k % s.db_in);
      src += buf;
    }
  };
  auto split_input = [&](int k) {
    if (splitd[k]) return;
    splitd[k] = 1;
    for (int l = 0; l < NL; ++l) {
      std::snprintf(buf, sizeof buf, "    float h%d_%d, l%d_%d; qsgb_split_f64(x%d%s, h%d_%d, l%d_%d, fb);\n", k, l, k,
                    l, k, lanes[l], k, l, k, l);
      src += buf;
    }
  };
  for (int r = 0; r < s.kout; ++r) {
    std::snprintf(buf, sizeof buf, "    V y%d;\n", r);
    src += buf;
  }
  // loads run `lookahead` inputs ahead of their first use
  std::vector<int> seq, pos(s.kin, 0);
  {
    std::vector<char> seen(s.kin, 0);
    for (int r : order)
      for (int k : s.cols[r])
        if (!seen[k]) {
          seen[k] = 1;
          pos[k] = (int)seq.size();
          seq.push_back(k);
        }
  }
  size_t lp = 0;
  auto load_upto = [&](size_t n) {
    for (; lp < seq.size() && lp < n; ++lp) load(seq[lp]);
  };
  load_upto((size_t)s.lookahead);
  if (s.lookahead >= s.kin) {  // small items: everything loaded and split up front
    for (int r = 0; r < s.kout; ++r)
      if (s.mode[r] == kModeDF)
        for (int k : s.cols[r]) split_input(k);
  }
  for (int r : order) {
    const int ra = r / s.db_out, rb = r % s.db_out;
    const auto& cols = s.cols[r];
    size_t need = 0;
    for (int k : cols) need = std::max(need, (size_t)pos[k] + 1);
    load_upto(need + (size_t)s.lookahead);
    for (int k : cols) {
      load(k);
      if (s.mode[r] == kModeDF) split_input(k);
    }
    const int ci = ci0[r];
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
        std::snprintf(buf, sizeof buf, "      fb |= qsgb_df_suspect(s%d);\n", l);
        src += buf;
        vals[l] = "qsgb_df_to_double(s" + std::to_string(l) + ", c" + std::to_string(l) + ")";
      }
    }
    if (s.pair) {
      src += "      y" + std::to_string(r) + ".x = " + vals[0] + "; y" + std::to_string(r) + ".y = " + vals[1] + ";\n";
    } else {
      src += "      y" + std::to_string(r) + " = " + vals[0] + ";\n";
    }
    src += "    }\n";
    done[r] = 1;
    if (s.stage_warps) {
      // results go to the tile once every row of the component (every row,
      // when all inputs were loaded first) is done
      pending.push_back(r);
      if (comp_last[r]) {
        for (int q : pending) {
          std::snprintf(buf, sizeof buf, "    t[lane * %d + %d] = y%d;\n", KS, q, q);
          src += buf;
        }
        pending.clear();
      }
    } else if (s.vout > 1) {
      const int r0 = r - r % s.vout;
      bool full = true;
      for (int j = 0; j < s.vout; ++j) full &= done[r0 + j] != 0;
      if (full) {
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
  if (s.stage_warps) {
    src += fallback;
    src += "    __syncwarp();\n";
    if (s.stage_bulk) {
      // generic-proxy tile writes -> visible to the bulk (async-proxy) store
      std::snprintf(buf, sizeof buf,
                    "    if (bulk) {\n"
                    "      asm volatile(\"fence.proxy.async.shared::cta;\" ::: \"memory\");\n"
                    "      __syncwarp();\n"
                    "      if (lane == 0) {\n"
                    "        asm volatile(\"cp.async.bulk.global.shared::cta.bulk_group [%%0], [%%1], %%2;\" :: "
                    "\"l\"(out + wt * %du), \"r\"(tb), \"r\"(nbytes) : \"memory\");\n"
                    "        asm volatile(\"cp.async.bulk.commit_group;\" ::: \"memory\");\n"
                    "      }\n"
                    "    } else {\n",
                    32 * KS);
      src += buf;
    }
    std::snprintf(buf, sizeof buf,
                  "    qsgb_i64 dstj[%d];\n"
                  "#pragma unroll\n"
                  "    for (int j = 0; j < %d; ++j) dstj[j] = __shfl_sync(0xffffffffu, bo, (lane + 32u * j) / %du);\n"
                  "#pragma unroll 1\n"
                  "    for (int ra = 0; ra < %d; ++ra) {\n"
                  "#pragma unroll\n"
                  "      for (int j = 0; j < %d; ++j) {\n"
                  "        const unsigned f = lane + 32u * j, i = f / %du, rb = f - i * %du;\n"
                  "        if (i < nv) out[dstj[j] + ra * p.h.sao + rb] = t[i * %d + ra * %d + rb];\n"
                  "      }\n"
                  "    }\n"
                  "%s"
                  "    __syncwarp();\n"
                  "  }\n",
                  s.db_out, s.db_out, s.db_out, s.kout / s.db_out, s.db_out, s.db_out, s.db_out, KS, s.db_out,
                  s.stage_bulk ? "    }\n" : "");
    src += buf;
    if (s.stage_bulk) src += "  if (lane == 0) asm volatile(\"cp.async.bulk.wait_group 0;\" ::: \"memory\");\n";
    src += "}\n";
  } else {
    src += fallback;
    src += "  }\n}\n";
  }
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

// ------------------------------------------------------------------ planning
// Row modes for the specialised kernel under QSGB_ARITH_AUTO: rows in
// ascending term count are computed in FP64 while that lowers the combined
// estimated times per group (SM clock cycles) of HBM traffic, the FP64
// pipe (kDpRate ops/clk), the integer pipe (64 lanes/clk: ~16 ops per split
// input, ~30 per float-float row result) and instruction issue (128/clk;
// ~12 per float-float term).
//
// The FP64 pipe sustains ~1.6-1.9 FMA/clk per SM (kDpRate).  Two-qubit
// PTMs denser than 2.5 terms per row are credited with kDpRateDense: the
// fused passes of the 14-qubit circuit (3-7 terms per row) left the FP64
// pipe 36-42 % busy while issue sat at 72-78 %, and moving more of their
// rows to FP64 took that circuit from 0.3053 to 0.2970 s (2.4: 0.2981 s).
// The same credit on every PTM cost 18 % on one-qubit rotations and 17 %
// on the 9x9 qutrit rotation.
constexpr double kDpRate = 1.6;
constexpr double kDpRateDense = 3.2;
void plan_modes(const std::vector<std::vector<int>>& cols, int kin, int arith, size_t esz, std::vector<int>& mode) {
  const int kout = (int)cols.size();
  mode.assign(kout, kModeZero);
  for (int r = 0; r < kout; ++r) {
    const int n = (int)cols[r].size();
    if (n == 0) continue;
    if (arith == QSGB_ARITH_F32) mode[r] = kModeF32;
    else if (arith == QSGB_ARITH_F64 || n == 1) mode[r] = kModeDP;
    else mode[r] = kModeDF;
  }
  if (arith != QSGB_ARITH_AUTO) return;
  std::vector<int> order;
  for (int r = 0; r < kout; ++r)
    if (cols[r].size() > 1) order.push_back(r);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cols[a].size() < cols[b].size(); });
  // Sparse PTMs (up to 3 terms per row) stream at close to the HBM rate,
  // where the float-float work overlaps memory worse than the estimate
  // says: weighting it twice moves more rows to the FP64 pipe.  Measured on
  // GB300, 14 qubits: noisy-CZ steps 1487 -> 1540 apps/s (6.3 -> 6.5 TB/s
  // per launch), rotation on qubit 5 5780 -> 6196 GB/s; the same weight on
  // dense PTMs lost 17 % (16x16: 1609 -> 1341 GB/s), so they keep 1.
  size_t n_terms = 0;
  for (const auto& c : cols) n_terms += c.size();
  const double sparse_bias = n_terms <= 3 * (size_t)kout ? 2.0 : 1.0;
  const double dp_rate = (kin == 16 && kout == 16 && (double)n_terms > 2.5 * kout) ? kDpRateDense : kDpRate;
  auto cost = [&](const std::vector<int>& m) {
    double dp = 0, alu = 0, issue = 0;
    std::vector<char> split(kin, 0);
    int n_used = 0;
    std::vector<char> used(kin, 0);
    for (int r = 0; r < kout; ++r) {
      for (int k : cols[r]) {
        if (!used[k]) {
          used[k] = 1;
          ++n_used;
        }
        if (m[r] == kModeDF) split[k] = 1;
      }
      if (m[r] == kModeDP) {
        dp += (double)cols[r].size();
        issue += (double)cols[r].size();
      } else if (m[r] == kModeDF) {
        issue += 12.0 * cols[r].size() + 30.0;
        alu += 30.0;
      }
    }
    for (int k = 0; k < kin; ++k)
      if (split[k]) {
        alu += 16.0;
        issue += 16.0;
      }
    issue += 2.0 * (n_used + kout);
    const double hbm = (double)(kin + kout) * (double)esz / 23.0;
    // the four times overlap imperfectly: a 6-norm rather than their maximum
    // (measured on GB300: 9x9 qutrit PTM 4853 -> 5539 GB/s, dense 16x16 and
    // the qubit PTMs unchanged)
    auto p6 = [](double t) { return t * t * t * t * t * t; };
    return std::pow(p6(hbm) + p6(dp / dp_rate) + p6(sparse_bias * alu / 64.0) + p6(sparse_bias * issue / 128.0),
                    1.0 / 6.0);
  };
  std::vector<int> m = mode;
  double best = cost(m);
  std::vector<int> best_m = m;
  for (int r : order) {
    m[r] = kModeDP;
    const double c = cost(m);
    if (c < best * 0.999) {
      best = c;
      best_m = m;
    }
  }
  mode = best_m;
}

}  // namespace

int Spec::n_coef() const {
  int n = 0;
  for (const auto& c : cols) n += (int)c.size();
  return n;
}

// How many inputs the generated loads run ahead of their first use.  Items
// of up to 36 values (16x16 pairs, 9x9) load everything first and compute
// rows in natural order; larger ones (81x81) go component by component with
// loads a few inputs ahead, which keeps them near 80-100 registers instead
// of 255.  Measured on GB300 (GB/s, 14 qubits / 8 qutrits): everything first
// gives noisy CZ 6354 and 81x81 on (2, 5) 2477; components with lookahead 8
// give 6326 and 4863; lookahead 16 to 255 lose up to 18 % on the CZ pair
// kernel.  On the 81x81 leakage CZ of 8 qutrits ((2, 5), (0, 1), (3, 4)),
// lookahead 4 / 6 / 8 / 9 / 10 / 11 / 12 / 16 / 32 / 81 gave about
// 4400 / 4830 / 5000 / 5190 / 5230 / 5250 / 4400 / 4870 / 3260 / 2810 GB/s:
// 9 to 11 is a plateau before a cliff at 12.
int lookahead_for(int kin, bool pair) { return kin * (pair ? 2 : 1) <= 36 ? kin : 10; }

bool make_spec(const double* ptm_host, int da_out, int db_out, int da_in, int db_in, int layout, int dtype,
               int arith, bool pair, bool z1, bool contiguous, int vin, int vout, Spec& spec,
               std::vector<double>& coef) {
  const int kin = da_in * db_in, kout = da_out * db_out;
  if (kin > 81 || kout > 81) return false;
  // op matrix M[r][k] from the stored layout (the generic kernel's ptm_index)
  std::vector<double> M((size_t)kin * kout);
  double amax = 0.0;
  for (int r = 0; r < kout; ++r)
    for (int k = 0; k < kin; ++k) {
      const int ra = r / db_out, rb = r % db_out;
      const int ka = k / db_in, kb = k % db_in;
      int idx;
      switch (layout & 3) {
        case 0: idx = r * kin + k; break;
        case QSGB_PTM_SWAPPED: idx = ((rb * da_out + ra) * db_in + kb) * da_in + ka; break;
        case QSGB_PTM_TRANSPOSED: idx = k * kout + r; break;
        default: idx = ((kb * da_in + ka) * db_out + rb) * da_out + ra; break;
      }
      const double v = ptm_host[idx];
      M[(size_t)r * kin + k] = v;
      amax = std::max(amax, std::fabs(v));
    }
  // float-float rows carry PTM entries as float pairs: a PTM whose largest
  // entry is outside [2^-100, 2^100] is computed in native FP64 throughout
  if (arith != QSGB_ARITH_F32 && !(amax >= 0x1p-100 && amax <= 0x1p100)) arith = QSGB_ARITH_F64;
  const double thr = arith == QSGB_ARITH_F64 ? 0.0 : amax * (arith == QSGB_ARITH_F32 ? 0x1p-30 : 0x1p-52);
  spec.kin = kin;
  spec.kout = kout;
  spec.db_in = db_in;
  spec.db_out = db_out;
  spec.pair = pair;
  spec.f32 = dtype == QSGB_F32;
  spec.vin = vin;
  spec.vout = vout;
  spec.lookahead = lookahead_for(kin, pair);
  spec.cols.assign(kout, {});
  for (int r = 0; r < kout; ++r)
    for (int k = 0; k < kin; ++k)
      if (std::fabs(M[(size_t)r * kin + k]) > thr) spec.cols[r].push_back(k);
  if (spec.n_coef() > kMaxJitTerms) return false;
  plan_modes(spec.cols, kin, arith, dtype == QSGB_F64 ? 8 : 4, spec.mode);
  // Z == 1 without full vector accesses on both sides: stage through shared
  // memory, as many warps per block as fit 48 KB of tiles (at most 4)
  spec.stage_warps = 0;
  spec.stage_bulk = false;
  // (measured on GB300: staging instead of 32-byte vector accesses loses 20 %
  // on a 16x16 PTM on the last two qubits, 5453 -> 4324 GB/s)
  if (z1 && !pair && (vin == 1 || vout == 1) && staged_in_place_ok(spec)) {
    const int tile = 32 * std::max(kin, kout) * (dtype == QSGB_F64 ? 8 : 4);
    spec.stage_warps = std::max(1, std::min(4, 49152 / tile));
    spec.stage_bulk = contiguous && kin == kout;
    spec.vin = spec.vout = 1;
  }
  coef.clear();
  coef.reserve(spec.n_coef());
  for (int r = 0; r < kout; ++r)
    for (int k : spec.cols[r]) {
      const double v = M[(size_t)r * kin + k];
      if (spec.mode[r] == kModeDF) {
        const float h = (float)v;
        const float l = (float)(v - (double)h);
        uint64_t bits = ((uint64_t)__builtin_bit_cast(uint32_t, h) << 32) | __builtin_bit_cast(uint32_t, l);
        coef.push_back(__builtin_bit_cast(double, bits));
      } else if (spec.mode[r] == kModeF32) {
        uint64_t bits = __builtin_bit_cast(uint32_t, (float)v);
        coef.push_back(__builtin_bit_cast(double, bits));
      } else {
        coef.push_back(v);
      }
    }
  return true;
}

std::string source(const Spec& s) { return gen_source(s); }

bool available() { return nvrtc().ok && !std::getenv("QSGB_NO_JIT"); }

// In-process cache key: everything gen_source reads, one byte per field (all
// values are below 256), so a cached pattern costs no code generation.
std::string spec_key(const Spec& s) {
  std::string k;
  k.reserve(8 + 2 * s.kout + s.n_coef());
  for (int v : {s.kin, s.kout, s.db_in, s.db_out, (int)s.pair, (int)s.f32, s.vin, s.vout, s.lookahead,
                s.stage_warps, (int)s.stage_bulk})
    k.push_back((char)v);
  for (int r = 0; r < s.kout; ++r) {
    k.push_back((char)s.mode[r]);
    k.push_back((char)s.cols[r].size());
    for (int c : s.cols[r]) k.push_back((char)c);
  }
  return k;
}

int kernel_for(const Spec& s, cudaKernel_t* k, std::string* src_out) {
  if (s.n_coef() > kMaxCoef) return QSGB_ERR_UNSUPPORTED;
  if (src_out) *src_out = gen_source(s);
  const std::string key = spec_key(s);
  Cache& c = cache();
  {
    std::lock_guard<std::mutex> g(c.mu);
    auto it = c.kernels.find(key);
    if (it != c.kernels.end()) {
      *k = it->second;
      return QSGB_OK;
    }
    if (c.failed.count(key)) return QSGB_ERR_UNSUPPORTED;
  }
  cudaKernel_t kern;
  const int st = compile(src_out ? *src_out : gen_source(s), &kern);
  std::lock_guard<std::mutex> g(c.mu);
  if (st != QSGB_OK) {
    c.failed[key] = st;
    return QSGB_ERR_UNSUPPORTED;
  }
  c.kernels[key] = kern;
  *k = kern;
  return QSGB_OK;
}

int prepare(const Spec& s) {
  cudaKernel_t kern;
  return kernel_for(s, &kern, nullptr);
}

int compile_only(const Spec& s, std::string* src_out) {
  if (s.n_coef() > kMaxCoef) return QSGB_ERR_UNSUPPORTED;
  const std::string src = gen_source(s);
  if (src_out) *src_out = src;
  Nvrtc& n = nvrtc();
  if (!n.ok) return QSGB_ERR_UNSUPPORTED;
  nvrtcProgram prog;
  if (n.create(&prog, src.c_str(), "qsgb_jit.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) return QSGB_ERR_UNSUPPORTED;
  const char* opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "-default-device"};
  const nvrtcResult cr = n.compile(prog, 3, opts);
  if (cr != NVRTC_SUCCESS && std::getenv("QSGB_JIT_VERBOSE")) {
    size_t ls = 0;
    n.log_size(prog, &ls);
    std::string log(ls, '\0');
    n.log(prog, &log[0]);
    std::fprintf(stderr, "qsgb jit: compilation failed:\n%s\n", log.c_str());
  }
  n.destroy(&prog);
  return cr == NVRTC_SUCCESS ? QSGB_OK : QSGB_ERR_CUDA;
}

namespace {

void fill_header(Hdr& h, const Geometry& g) {
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
}

// The parameter block (header + coefficients) is assembled in `blob`.
int launch_blob(cudaKernel_t kern, const Spec& s, const Geometry& g, unsigned char* blob, cudaStream_t stream) {
  Hdr h;
  fill_header(h, g);
  std::memcpy(blob, &h, sizeof h);
  void* args[] = {blob};
  const unsigned block = s.stage_warps ? 32u * (unsigned)s.stage_warps : 128u;
  const uint64_t need = (g.n_items + block - 1) / block;
  const uint64_t cap = (uint64_t)sm_count() * 16;
  const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min(need, cap));
  QSGB_CUDA_TRY(cudaLaunchKernel((const void*)kern, dim3(grid), dim3(block), args, 0, stream));
  return QSGB_OK;
}

struct FastKeyHash {
  size_t operator()(const FastKey& k) const {
    unsigned long long h = 1469598103934665603ull;
    for (unsigned char c : k.hdr) h = (h ^ c) * 1099511628211ull;
    for (int i = 0; i < k.nwords; ++i) h = (h ^ k.mask[i]) * 1099511628211ull;
    return (size_t)h;
  }
};

struct FastCache {
  std::mutex mu;
  std::unordered_map<FastKey, FastEntry, FastKeyHash> map;
};
FastCache& fast_cache() {
  static FastCache c;
  return c;
}

}  // namespace

bool FastKey::operator==(const FastKey& o) const {
  if (nwords != o.nwords || std::memcmp(hdr, o.hdr, sizeof hdr) != 0) return false;
  return std::memcmp(mask, o.mask, sizeof(unsigned long long) * (size_t)nwords) == 0;
}

const FastEntry* fast_find(const FastKey& key) {
  FastCache& c = fast_cache();
  std::lock_guard<std::mutex> g(c.mu);
  auto it = c.map.find(key);
  return it == c.map.end() ? nullptr : &it->second;  // entries are never erased
}

const FastEntry* fast_insert(const FastKey& key, const Spec& spec, int layout, int da_out, int db_out, int da_in,
                             int db_in) {
  FastEntry e;
  if (kernel_for(spec, &e.kern, nullptr) != QSGB_OK) return nullptr;
  e.spec = spec;
  const int kin = da_in * db_in, kout = da_out * db_out;
  for (int r = 0; r < spec.kout; ++r)
    for (int k : spec.cols[r]) {
      const int ra = r / db_out, rb = r % db_out, ka = k / db_in, kb = k % db_in;
      int idx;
      switch (layout & 3) {
        case 0: idx = r * kin + k; break;
        case QSGB_PTM_SWAPPED: idx = ((rb * da_out + ra) * db_in + kb) * da_in + ka; break;
        case QSGB_PTM_TRANSPOSED: idx = k * kout + r; break;
        default: idx = ((kb * da_in + ka) * db_out + rb) * da_out + ra; break;
      }
      e.src.push_back(idx);
      e.kind.push_back((unsigned char)spec.mode[r]);
    }
  FastCache& c = fast_cache();
  std::lock_guard<std::mutex> g(c.mu);
  auto it = c.map.emplace(key, std::move(e)).first;
  return &it->second;
}

int launch_entry(const FastEntry& e, const Geometry& g, const double* ptm_host, cudaStream_t stream) {
  // header + coefficients, at most 32764 bytes (kMaxCoef)
  alignas(16) unsigned char blob[sizeof(Hdr) + 8 * (size_t)kMaxCoef];
  double* coef = reinterpret_cast<double*>(blob + sizeof(Hdr));
  const size_t n = e.src.size();
  for (size_t t = 0; t < n; ++t) {
    const double v = ptm_host[e.src[t]];
    if (e.kind[t] == kModeDF) {
      const float h = (float)v;
      const float l = (float)(v - (double)h);
      const uint64_t bits = ((uint64_t)__builtin_bit_cast(uint32_t, h) << 32) | __builtin_bit_cast(uint32_t, l);
      coef[t] = __builtin_bit_cast(double, bits);
    } else if (e.kind[t] == kModeF32) {
      coef[t] = __builtin_bit_cast(double, (uint64_t)__builtin_bit_cast(uint32_t, (float)v));
    } else {
      coef[t] = v;
    }
  }
  if (n == 0) coef[0] = 0.0;
  return launch_blob(e.kern, e.spec, g, blob, stream);
}

int launch(const Spec& s, const Geometry& g, const double* coef, cudaStream_t stream) {
  cudaKernel_t kern;
  const int st = kernel_for(s, &kern, nullptr);
  if (st != QSGB_OK) return st;
  const int nc = std::max(1, s.n_coef());
  std::vector<unsigned char> blob(sizeof(Hdr) + 8 * (size_t)nc, 0);
  std::memcpy(blob.data() + sizeof(Hdr), coef, 8 * (size_t)s.n_coef());
  return launch_blob(kern, s, g, blob.data(), stream);
}

}  // namespace jit
}  // namespace qsgb

extern "C" int qsgb_jit_available(void) { return qsgb::jit::available() ? 1 : 0; }
