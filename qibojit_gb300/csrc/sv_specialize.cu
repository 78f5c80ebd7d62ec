// sv_specialize.cu -- pass kernels compiled at run time for one program's structure.
//
// The tile kernel of sv_fused.cu interprets a pass: every phase and op is decoded
// from the kernel parameters, register positions go through switch tables, shared-
// memory offsets are loaded per amplitude.  For a program that runs many times (the
// same circuit with new parameters, or repeated shots of one circuit) the engine can
// instead emit CUDA C++ for each pass with all of that fixed: tile and register bit
// positions, offsets, op order and kinds, control masks and sign tables become
// literals, and the gate coefficients are read straight from the kernel parameters.
// The source is compiled for sm_103a by the CUDA runtime compiler (NVRTC, loaded
// with dlopen so the library has no link-time dependency on it), loaded with
// cudaLibraryLoadData and launched like the interpreted pass: same tiles, same
// double-buffered cp.async staging, same register ops (sv_device.cuh, whose text is
// compiled into this library).  Compiled kernels are cached per process by their
// source text, which holds no coefficient values, and their cubins on disk.
#include <dlfcn.h>
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <type_traits>
#include <condition_variable>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "sv_plan.cuh"
#include "sv_device_text.inc"  // kDeviceHeaderText: sv_device.cuh as a string (generated at build time)

namespace sv {

// ------------------------------------------------------------- NVRTC (dlopen)
namespace {

typedef int nvrtcResult_t;
typedef struct _nvrtcProgram* nvrtcProgram_t;

struct Nvrtc {
  void* handle = nullptr;
  nvrtcResult_t (*create)(nvrtcProgram_t*, const char*, const char*, int, const char* const*,
                          const char* const*) = nullptr;
  nvrtcResult_t (*compile)(nvrtcProgram_t, int, const char* const*) = nullptr;
  nvrtcResult_t (*destroy)(nvrtcProgram_t*) = nullptr;
  nvrtcResult_t (*log_size)(nvrtcProgram_t, size_t*) = nullptr;
  nvrtcResult_t (*log)(nvrtcProgram_t, char*) = nullptr;
  nvrtcResult_t (*cubin_size)(nvrtcProgram_t, size_t*) = nullptr;
  nvrtcResult_t (*cubin)(nvrtcProgram_t, char*) = nullptr;
  nvrtcResult_t (*version)(int*, int*) = nullptr;
  bool ok = false;
};

const Nvrtc& nvrtc() {
  static Nvrtc api;
  static std::once_flag once;
  std::call_once(once, [] {
    const char* names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13",
                           "/usr/local/cuda/lib64/libnvrtc.so"};
    for (const char* nm : names) {
      api.handle = dlopen(nm, RTLD_NOW | RTLD_LOCAL);
      if (api.handle) break;
    }
    if (!api.handle) return;
    auto sym = [](const char* s) { return dlsym(api.handle, s); };
    api.create = (decltype(api.create))sym("nvrtcCreateProgram");
    api.compile = (decltype(api.compile))sym("nvrtcCompileProgram");
    api.destroy = (decltype(api.destroy))sym("nvrtcDestroyProgram");
    api.log_size = (decltype(api.log_size))sym("nvrtcGetProgramLogSize");
    api.log = (decltype(api.log))sym("nvrtcGetProgramLog");
    api.cubin_size = (decltype(api.cubin_size))sym("nvrtcGetCUBINSize");
    api.cubin = (decltype(api.cubin))sym("nvrtcGetCUBIN");
    api.version = (decltype(api.version))sym("nvrtcVersion");
    api.ok = api.create && api.compile && api.destroy && api.log_size && api.log && api.cubin_size && api.cubin;
  });
  return api;
}

// ---------------------------------------------------------------- generator
// `var`'s bit i moved to bit pos[i], as one shift-and-mask term per run of consecutive positions
std::string deposit_expr(const char* var, const std::vector<int>& pos, bool wide) {
  std::ostringstream o;
  size_t i = 0;
  bool first = true;
  while (i < pos.size()) {
    size_t j = i + 1;
    while (j < pos.size() && pos[j] == pos[j - 1] + 1) j++;
    const long long mask = (1ll << (j - i)) - 1;
    o << (first ? "" : " | ") << "((" << (wide ? "(long long)" : "") << "(" << var << " >> " << i << ") & " << mask
      << (wide ? "ll" : "") << ") << " << pos[i] << ")";
    first = false;
    i = j;
  }
  if (first) o << "0";
  return o.str();
}

// Shared-memory bank slot of tile element e in the padded tile layout (smem_pos), for
// elements of `esize` bytes (a 128-byte bank row holds 128/esize slots).
static int bank_slot(int e, int esize) { return smem_pos(e) % (128 / esize); }

// Order of a phase's non-register tile bits for the thread-bit deposit: the first five
// (a warp's lanes) are chosen so that the warp's 32 shared-memory accesses of one
// register spread evenly over the bank slots (the ascending order can put two lanes
// bits on the same slot weight, e.g. bits 3 and 7, doubling the wavefronts); the rest
// stay ascending.  Loads, stores and thread-level masks of the phase all derive from
// the same deposit, so any order is correct.
std::vector<int> lane_order(const std::vector<int>& nonreg, int esize) {
  if (nonreg.size() <= 5) return nonreg;
  const int slots = 128 / esize;
  auto cost = [&](const std::vector<int>& lanes) {
    std::vector<int> hits(slots, 0);
    int worst = 0;
    for (int L = 0; L < 32; L++) {
      int e = 0;
      for (int i = 0; i < 5; i++)
        if ((L >> i) & 1) e |= 1 << lanes[i];
      worst = std::max(worst, ++hits[bank_slot(e, esize)]);
    }
    return worst;
  };
  std::vector<int> best(nonreg.begin(), nonreg.begin() + 5);
  int best_cost = cost(best);
  const int m = (int)nonreg.size();
  for (int a = 0; a < m && best_cost > 32 / slots; a++)
    for (int b = a + 1; b < m; b++)
      for (int c = b + 1; c < m; c++)
        for (int d = c + 1; d < m; d++)
          for (int f = d + 1; f < m; f++) {
            const std::vector<int> cand = {nonreg[a], nonreg[b], nonreg[c], nonreg[d], nonreg[f]};
            const int k = cost(cand);
            if (k < best_cost) {
              best_cost = k;
              best = cand;
            }
          }
  std::vector<int> out = best;
  for (int b : nonreg)
    if (std::find(best.begin(), best.end(), b) == best.end()) out.push_back(b);
  return out;
}

int coef_count(const FOp& f) {
  switch (f.type) {
    case FOP_D1RUN:
    case FOP_D1RUNR: return (int)f.coef + 4 * f.nrun;
    case FOP_DIAGR: return (int)f.coef + 16;
    case FOP_DENSE1:
    case FOP_DENSE1R: return (int)f.coef + 4;
    case FOP_DENSE1P: return (int)f.coef + 2;
    case FOP_DENSE2: return (int)f.coef + 16;
    case FOP_DIAG: return (int)f.coef + (1 << f.nd);
    default: return 0;
  }
}

struct KernelShape {
  int threads, maxt, minb;
  size_t smem;
};

// what a generated pass kernel runs over: one state, a batch of states, or the
// adjoint sweep's psi and lambda states of a batch together with gradient markers
enum PassMode { PASS_SINGLE = 0, PASS_BATCHED = 1, PASS_ADJOINT = 2 };

// gradient slots an adjoint pass accumulates into (the markers' slot numbers)
template <typename T>
int adjoint_slots(const PassParams<T>& p) {
  int ng = 0;
  for (int q = 0; q < p.nops; q++) {
    const FOp& f = p.ops[q];
    if (f.type == FOP_GRADX || f.type == FOP_GRADY || f.type == FOP_GRADZ) ng = std::max(ng, (int)f.u1 + 1);
  }
  return ng;
}

template <typename T>
KernelShape shape_of(int kt, int mode = PASS_SINGLE, int nslots = 0) {
  KernelShape k;
  k.threads = 1 << (kt - kRB);
  if (mode == PASS_ADJOINT) {
    // psi and lambda tiles, both double-buffered, one FP64 sum per marker and the
    // current tile's warp sums (the state's real type) per marker and warp
    k.smem = 4 * sizeof(T) * (size_t)tile_stride(1 << kt) + sizeof(double) * (size_t)nslots +
             sizeof(T) / 2 * (size_t)nslots * (k.threads / 32);
    k.maxt = k.threads;
    k.minb = (int)std::max<size_t>(1, std::min<size_t>(8, (size_t)(227 * 1024) / k.smem));
    return k;
  }
  k.maxt = k.threads <= 256 ? 256 : 512;
  k.minb = (sizeof(T) < 16 && k.threads <= 256) ? 3 : 1;  // the interpreted pass's launch variants
  k.smem = 2 * sizeof(T) * (size_t)tile_stride(1 << kt);
  return k;
}

// CUDA source of one pass: kernel `name`, coefficients in a by-value parameter struct.
// A batched pass (a group of circuits of one structure) runs over (circuit, tile) items
// instead, with each circuit's state from a pointer table and its coefficients from its
// block of a device array (coef_stride elements apart, the pass's own at coef_goff).
// An adjoint pass is a batched pass over two states per circuit, psi and lambda, that
// applies every op to both and evaluates the gradient markers between them: each
// marker's Im<lambda|G|psi> is summed over a warp and then over the tile's warps in
// the state's precision, over tiles in an FP64 shared-memory slot (one FP64 add per
// marker and tile), and written per block and circuit to gpart (the interpreted
// adjoint pass's layout).
template <typename T>
std::string pass_source(const PassParams<T>& p, const char* name, int mode = PASS_SINGLE) {
  const bool batched = mode != PASS_SINGLE, adj = mode == PASS_ADJOINT;
  if (adj && stored_as_double_pairs<T>::value) return std::string();  // adjoint: complex64 and complex128 only
  std::ostringstream o;
  const char* ty = stored_as_double_pairs<T>::value ? "sv::cw" : (sizeof(T) == 16 ? "sv::c128" : "sv::c64");
  // double-word passes convert the tile to float pairs in place once it has arrived
  const char* conv = stored_as_double_pairs<T>::value
                         ? "#pragma unroll\n    for (int k = 0; k < 16; k++) sv::cw_from_stored(tile + stid + POSK[k]);\n"
                           "    __syncthreads();\n"
                         : "";
  const int kt = p.kt, n = p.n;
  const int nslots = adj ? adjoint_slots(p) : 0;
  const KernelShape ks = shape_of<T>(kt, mode, nslots);
  const int nth = ks.threads;
  int ncoef = 1;
  for (int q = 0; q < p.nops; q++) ncoef = std::max(ncoef, coef_count(p.ops[q]));
  std::vector<int> tpos(p.tile_pos, p.tile_pos + kt), outer;
  for (int g = 0; g < n; g++)
    if (std::find(tpos.begin(), tpos.end(), g) == tpos.end()) outer.push_back(g);
  const std::vector<int> low(tpos.begin(), tpos.begin() + (kt - kRB));
  const char* CF = batched ? "C" : "cf.c";  // where the ops read their coefficients
  if (adj)
    o << "extern \"C\" __global__ void __launch_bounds__(" << ks.maxt << ", " << ks.minb << ") " << name << "(" << ty
      << "* const* __restrict__ psis, " << ty << "* const* __restrict__ lams, const " << ty
      << "* __restrict__ coefs, long long coef_stride, int ncirc, double* __restrict__ gpart, int nparams, "
         "int gstride) {\n";
  else if (batched)
    o << "extern \"C\" __global__ void __launch_bounds__(" << ks.maxt << ", " << ks.minb << ") " << name << "(" << ty
      << "* const* __restrict__ states, const " << ty << "* __restrict__ coefs, long long coef_stride, int ncirc) {\n";
  else
    o << "struct " << name << "_coef { " << ty << " c[" << ncoef << "]; };\n"
      << "extern \"C\" __global__ void __launch_bounds__(" << ks.maxt << ", " << ks.minb << ") " << name << "(" << ty
      << "* __restrict__ state, const __grid_constant__ " << name << "_coef cf) {\n";
  o << "  using T = " << ty << ";\n"
    << "  extern __shared__ __align__(16) unsigned char smem_raw[];\n"
    << "  T* const buf0 = reinterpret_cast<T*>(smem_raw);\n"
    << "  constexpr int TSTRIDE = " << tile_stride(1 << kt) << ";\n"
    << "  const int tid = threadIdx.x;\n"
    // tile element e = tid + k * threads: its low bits are tid's, its top four bits k's
    << "  const long long dtid = " << deposit_expr("tid", low, true) << ";\n"
    << "  const int stid = tid + (tid >> 4) + (tid >> 8);\n"
    << "  constexpr long long DEPK[16] = {";
  for (int k = 0; k < 16; k++) {
    long long d = 0;
    for (int i = 0; i < 4; i++)
      if ((k >> i) & 1) d |= 1ll << tpos[kt - kRB + i];
    o << d << "ll" << (k < 15 ? ", " : "};\n");
  }
  // shared-memory position of element tid + k * threads: smem_pos is additive over the
  // disjoint bits of tid and k * threads
  o << "  constexpr int POSK[16] = {";
  for (int k = 0; k < 16; k++) o << smem_pos(k * nth) << (k < 15 ? ", " : "};\n");
  if (adj) {
    const int tshift = n - kt;
    o << "  using R = sv::real_of<T>::type;\n"
      << "  constexpr int NW = " << nth / 32 << ";\n"
      << "  const int warp = tid >> 5, lane = tid & 31;\n"
      << "  (void)warp;\n  (void)lane;\n";
    if (nslots > 0) {
      std::vector<int> param(nslots, -1);
      for (int q = 0; q < p.nops; q++) {
        const FOp& f = p.ops[q];
        if (f.type == FOP_GRADX || f.type == FOP_GRADY || f.type == FOP_GRADZ) param[f.u1] = (int)f.coef;
      }
      o << "  constexpr int NG = " << nslots << ";\n"
        << "  constexpr int PARAM[NG] = {";
      for (int g = 0; g < nslots; g++) o << param[g] << (g + 1 < nslots ? ", " : "};\n");
      o << "  double* const gacc = reinterpret_cast<double*>(buf0 + 4 * TSTRIDE);  // [slot]\n"
        << "  R* const gw = reinterpret_cast<R*>(gacc + NG);  // [slot][warp], the current tile's\n"
        << "  for (int i = tid; i < NG; i += " << nth << ") gacc[i] = 0.0;\n"
        << "  for (int i = tid; i < NG * NW; i += " << nth << ") gw[i] = 0;\n"
        << "  __syncthreads();\n"
        // a tile's warp sums into the FP64 slots (after the tile's last barrier)
        << "  auto add_tile = [&]() {\n"
        << "    for (int g = tid; g < NG; g += " << nth << ") {\n"
        << "      R s = gw[g * NW];\n"
        << "      for (int w = 1; w < NW; w++) s += gw[g * NW + w];\n"
        << "      gacc[g] += (double)s;\n"
        << "    }\n"
        << "  };\n"
        // this block's sums of one circuit, then the slots cleared
        << "  auto flush_grads = [&](int circ) {\n"
        << "    __syncthreads();\n"
        << "    for (int g = tid; g < NG; g += " << nth << ") {\n"
        << "      if (PARAM[g] >= 0) gpart[((long long)circ * nparams + PARAM[g]) * gstride + blockIdx.x] = gacc[g];\n"
        << "      gacc[g] = 0.0;\n"
        << "    }\n"
        << "    __syncthreads();\n"
        << "  };\n";
    } else {
      o << "  auto add_tile = [&]() {};\n"
        << "  auto flush_grads = [&](int) {};\n"
        << "  (void)gpart;\n  (void)nparams;\n  (void)gstride;\n";
    }
    o << "  const long long nitems = " << p.ntiles << "ll * ncirc;\n"
      << "  auto origin = [&](long long it) -> long long { const long long t = it & " << (p.ntiles - 1) << "ll; return "
      << deposit_expr("t", outer, true) << "; };\n"
      << "  auto issue_load = [&](int slot, long long it) {\n"
      << "    const long long base = origin(it);\n"
      << "    const T* const sp = psis[it >> " << tshift << "];\n"
      << "    const T* const sl = lams[it >> " << tshift << "];\n"
      << "#pragma unroll\n"
      << "    for (int k = 0; k < 16; k++) {\n"
      << "      sv::cp_async<sizeof(T)>(buf0 + slot * TSTRIDE + stid + POSK[k], sp + (base | dtid | DEPK[k]));\n"
      << "      sv::cp_async<sizeof(T)>(buf0 + (2 + slot) * TSTRIDE + stid + POSK[k], sl + (base | dtid | DEPK[k]));\n"
      << "    }\n"
      << "    sv::cp_async_commit();\n"
      << "  };\n"
      << "  long long t = blockIdx.x;\n"
      << "  if (t < nitems) issue_load(0, t);\n"
      << "  int cur = 0, cur_circ = -1;\n"
      << "  for (; t < nitems; t += gridDim.x, cur ^= 1) {\n"
      << "    const int circ = (int)(t >> " << tshift << ");\n"
      << "    if (circ != cur_circ) {\n"
      << "      if (cur_circ >= 0) flush_grads(cur_circ);\n"
      << "      cur_circ = circ;\n"
      << "    }\n"
      << "    T* const tile = buf0 + cur * TSTRIDE;\n"
      << "    T* const ltile = buf0 + (2 + cur) * TSTRIDE;\n"
      << "    const long long base = origin(t);\n"
      << "    const T* const C = coefs + (long long)circ * coef_stride + " << p.coef_goff << ";\n"
      << "    (void)C;\n"
      << "    const long long tn = t + gridDim.x;\n"
      << "    if (tn < nitems) {\n"
      << "      issue_load(cur ^ 1, tn);\n"
      << "      sv::cp_async_wait<1>();\n"
      << "    } else {\n"
      << "      sv::cp_async_wait<0>();\n"
      << "    }\n"
      << "    __syncthreads();\n";
  } else if (batched) {
    const int tshift = n - kt;
    o << "  const long long nitems = " << p.ntiles << "ll * ncirc;\n"
      << "  auto origin = [&](long long it) -> long long { const long long t = it & " << (p.ntiles - 1) << "ll; return "
      << deposit_expr("t", outer, true) << "; };\n"
      << "  auto item_state = [&](long long it) -> T* { return states[it >> " << tshift << "]; };\n"
      << "  auto issue_load = [&](T* buf, const T* sp, long long base) {\n"
      << "#pragma unroll\n"
      << "    for (int k = 0; k < 16; k++)\n"
      << "      sv::cp_async<sizeof(T)>(buf + stid + POSK[k], sp + (base | dtid | DEPK[k]));\n"
      << "    sv::cp_async_commit();\n"
      << "  };\n"
      << "  long long t = blockIdx.x;\n"
      << "  if (t < nitems) issue_load(buf0, item_state(t), origin(t));\n"
      << "  int cur = 0;\n"
      << "  for (; t < nitems; t += gridDim.x, cur ^= 1) {\n"
      << "    T* const tile = buf0 + cur * TSTRIDE;\n"
      << "    const long long base = origin(t);\n"
      << "    T* const st = item_state(t);\n"
      << "    const T* const C = coefs + (t >> " << tshift << ") * coef_stride + " << p.coef_goff << ";\n"
      << "    const long long tn = t + gridDim.x;\n"
      << "    if (tn < nitems) {\n"
      << "      issue_load(buf0 + (cur ^ 1) * TSTRIDE, item_state(tn), origin(tn));\n"
      << "      sv::cp_async_wait<1>();\n"
      << "    } else {\n"
      << "      sv::cp_async_wait<0>();\n"
      << "    }\n"
      << "    __syncthreads();\n" << conv;
  } else {
    o << "  const long long nitems = " << p.ntiles << "ll;\n"
      << "  auto origin = [&](long long t) -> long long { return " << deposit_expr("t", outer, true) << "; };\n"
      << "  auto issue_load = [&](T* buf, long long base) {\n"
      << "#pragma unroll\n"
      << "    for (int k = 0; k < 16; k++)\n"
      << "      sv::cp_async<sizeof(T)>(buf + stid + POSK[k], state + (base | dtid | DEPK[k]));\n"
      << "    sv::cp_async_commit();\n"
      << "  };\n"
      << "  long long t = blockIdx.x;\n"
      << "  if (t < nitems) issue_load(buf0, origin(t));\n"
      << "  int cur = 0;\n"
      << "  for (; t < nitems; t += gridDim.x, cur ^= 1) {\n"
      << "    T* const tile = buf0 + cur * TSTRIDE;\n"
      << "    const long long base = origin(t);\n"
      << "    const long long tn = t + gridDim.x;\n"
      << "    if (tn < nitems) {\n"
      << "      issue_load(buf0 + (cur ^ 1) * TSTRIDE, origin(tn));\n"
      << "      sv::cp_async_wait<1>();\n"
      << "    } else {\n"
      << "      sv::cp_async_wait<0>();\n"
      << "    }\n"
      << "    __syncthreads();\n" << conv;
  }
  // the register arrays every op applies to: the state, or psi and lambda
  const std::vector<std::string> arrs = adj ? std::vector<std::string>{"v", "w"} : std::vector<std::string>{"v"};
  for (int ph = 0; ph < p.nphases; ph++) {
    const Phase& P = p.phases[ph];
    std::vector<int> nonreg;
    for (int b = 0; b < kt; b++)
      if (b != P.rb[0] && b != P.rb[1] && b != P.rb[2] && b != P.rb[3]) nonreg.push_back(b);
    nonreg = lane_order(nonreg, (int)sizeof(T));
    o << "    {  // phase " << ph << ", register bits " << (int)P.rb[0] << " " << (int)P.rb[1] << " "
      << (int)P.rb[2] << " " << (int)P.rb[3] << "\n"
      << "      const int lbase = " << deposit_expr("tid", nonreg, false) << ";\n"
      << "      (void)lbase;\n"
      << "      T* const tp = tile + lbase + (lbase >> 4) + (lbase >> 8);\n"
      << "      T v[16];\n";
    for (int j = 0; j < 16; j++) o << "      v[" << j << "] = tp[" << P.soff[j] << "];\n";
    if (adj) {
      o << "      T* const tq = ltile + lbase + (lbase >> 4) + (lbase >> 8);\n"
        << "      T w[16];\n";
      for (int j = 0; j < 16; j++) o << "      w[" << j << "] = tq[" << P.soff[j] << "];\n";
    }
    bool uses_pn = false;
    for (int q = P.op_begin; q < P.op_end; q++) uses_pn |= p.ops[q].type == FOP_SIGN;
    if (uses_pn) o << "      unsigned pn = 0;\n";
    unsigned stat = 0;  // negations known at compile time
    bool dyn = false;   // run-time negations pending in pn
    auto flush = [&]() {
      for (int j = 0; j < 16; j++)
        if ((stat >> j) & 1)
          for (const std::string& a : arrs) o << "      " << a << "[" << j << "] = sv::tneg(" << a << "[" << j << "]);\n";
      stat = 0;
      if (dyn) {
        for (const std::string& a : arrs) o << "      sv::apply_negations(" << a << ", pn);\n";
        o << "      pn = 0;\n";
      }
      dyn = false;
    };
    // one statement per register array, under the op's condition when it has one
    auto each = [&](const std::string& pre, auto&& stmt) {
      if (arrs.size() == 1) {
        o << pre << stmt(arrs[0]) << "\n";
        return;
      }
      o << pre << "{\n";
      for (const std::string& a : arrs) o << "        " << stmt(a) << "\n";
      o << "      }\n";
    };
    // a gradient marker's warp sum, added to its FP64 slot by the warp's first lane
    auto grad_sum = [&](const FOp& f, const std::string& expr) {
      o << "      {\n        R g = " << expr << ";\n"
        << "#pragma unroll\n"
        << "        for (int off = 16; off > 0; off >>= 1) g += __shfl_xor_sync(0xffffffffu, g, off);\n"
        << "        if (lane == 0) gw[" << (int)f.u1 << " * NW + warp] = g;\n"
        << "      }\n";
    };
    // the thread / tile control test of an op, and the non-register part of a diagonal's
    // table index (empty when the op has none)
    auto cond_of = [](const FOp& f) {
      std::ostringstream c;
      if (f.type != FOP_D1RUN && f.type != FOP_D1RUNR && f.type != FOP_DIAGR) {
        if (f.omask) c << "((base & " << (long long)f.omask << "ll) == " << (long long)f.omask << "ll)";
        if (f.tmask) c << (f.omask ? " && " : "") << "((lbase & " << f.tmask << ") == " << f.tmask << ")";
      }
      return c.str();
    };
    auto index_of = [](const FOp& f) {
      std::ostringstream te;
      bool tany = false;
      for (int i = 0; i < f.nd; i++) {
        const int sh = f.nd - 1 - i;
        if (f.tb[i] >= 0) te << (tany ? " | " : "") << "(((lbase >> " << (int)f.tb[i] << ") & 1) << " << sh << ")";
        else if (f.ob[i] >= 0) te << (tany ? " | " : "") << "((int)((base >> " << (int)f.ob[i] << ") & 1) << " << sh << ")";
        else continue;
        tany = true;
      }
      return te.str();
    };
    // two diagonals whose factors depend on the registers in the same way
    auto same_shape = [](const FOp& a, const FOp& b) {
      if (a.jmask != b.jmask) return false;
      for (int j = 0; j < 16; j++)
        if (((a.jmask >> j) & 1) && ((a.rpart >> (4 * j)) & 15) != ((b.rpart >> (4 * j)) & 15)) return false;
      return true;
    };
    std::vector<char> consumed(P.op_end, 0);
    for (int q = P.op_begin; q < P.op_end; q++) {
      const FOp& f = p.ops[q];
      if (consumed[q]) continue;
      const std::string cond = cond_of(f);
      const std::string pre = cond.empty() ? "      " : "      if (" + cond + ") ";
      if (f.type == FOP_D1RUN || f.type == FOP_D1RUNR || f.type == FOP_DENSE1 || f.type == FOP_DENSE1R ||
          f.type == FOP_DENSE1P || f.type == FOP_X1 || f.type == FOP_SWAP2 || f.type == FOP_DENSE2 ||
          f.type == FOP_GRADX || f.type == FOP_GRADY)
        flush();
      const std::string tix = index_of(f);
      const bool tany = !tix.empty();
      std::ostringstream te;
      te << tix;
      const std::string cf = std::string(CF) + " + ";
      switch (f.type) {
        case FOP_D1RUN:
          for (int k = 0; k < f.nrun; k++)
            each("      ", [&](const std::string& a) {
              return "sv::dense1_regs<T, " + std::to_string((int)f.ru[k]) + ">(" + a + ", " + cf +
                     std::to_string(f.coef + 4 * k) + ", 0xffffu);";
            });
          break;
        case FOP_D1RUNR:
          for (int k = 0; k < f.nrun; k++)
            each("      ", [&](const std::string& a) {
              return "sv::dense1r_regs<T, " + std::to_string((int)f.ru[k]) + ">(" + a + ", " + cf +
                     std::to_string(f.coef + 4 * k) + ", 0xffffu);";
            });
          break;
        case FOP_DIAGR:  // commutes with the pending sign flips
          for (int j = 0; j < 16; j++)
            for (const std::string& a : arrs)
              o << "      " << a << "[" << j << "] = sv::tmul(" << CF << "[" << (f.coef + j) << "], " << a << "[" << j
                << "]);\n";
          break;
        case FOP_DENSE1:
          each(pre, [&](const std::string& a) {
            return "sv::dense1_regs<T, " + std::to_string((int)f.u0) + ">(" + a + ", " + cf + std::to_string(f.coef) +
                   ", " + std::to_string(f.jmask) + "u);";
          });
          break;
        case FOP_DENSE1P:
          each(pre, [&](const std::string& a) {
            return "sv::pivot1_regs<T, " + std::to_string((int)f.u0) + ", " + std::to_string((int)f.u1) + ">(" + a +
                   ", " + cf + std::to_string(f.coef) + ", " + std::to_string(f.jmask) + "u);";
          });
          break;
        case FOP_DENSE1R:
          each(pre, [&](const std::string& a) {
            return "sv::dense1r_regs<T, " + std::to_string((int)f.u0) + ">(" + a + ", " + cf + std::to_string(f.coef) +
                   ", " + std::to_string(f.jmask) + "u);";
          });
          break;
        case FOP_X1:
          each(pre, [&](const std::string& a) {
            return "sv::x1_regs<T, " + std::to_string((int)f.u0) + ">(" + a + ", " + std::to_string(f.jmask) + "u);";
          });
          break;
        case FOP_SWAP2:
          each(pre, [&](const std::string& a) {
            return "sv::swap2_regs<T, " + std::to_string((int)std::min(f.u0, f.u1)) + ", " +
                   std::to_string((int)std::max(f.u0, f.u1)) + ">(" + a + ", " + std::to_string(f.jmask) + "u);";
          });
          break;
        case FOP_DENSE2:
          each(pre, [&](const std::string& a) {
            return "sv::dense2_regs<T, " + std::to_string((int)f.u0) + ", " + std::to_string((int)f.u1) + ">(" + a +
                   ", " + cf + std::to_string(f.coef) + ", " + std::to_string(f.jmask) + "u);";
          });
          break;
        case FOP_SIGN:
          if (!tany && cond.empty()) {
            stat ^= f.neg[0];
          } else {
            unsigned long long lo = 0, hi = 0;
            for (int t2 = 0; t2 < 8; t2++) (t2 < 4 ? lo : hi) |= (unsigned long long)f.neg[t2] << (16 * (t2 & 3));
            o << pre << "{\n        const int ti = " << (tany ? te.str() : std::string("0")) << ";\n"
              << "        pn ^= (unsigned)(((ti < 4) ? (" << lo << "ull >> (16 * ti)) : (" << hi
              << "ull >> (16 * (ti - 4)))) & 0xffffull);\n      }\n";
            dyn = true;
          }
          break;
        case FOP_DIAG: {
          // this diagonal and the later ones of the same register shape up to the next
          // non-diagonal op commute: their factors multiply per thread first (one complex
          // multiply per distinct register index and op) and reach the amplitudes once
          std::vector<int> members{q};
          for (int q2 = q + 1; q2 < P.op_end && (p.ops[q2].type == FOP_DIAG || p.ops[q2].type == FOP_SIGN); q2++)
            if (p.ops[q2].type == FOP_DIAG && same_shape(p.ops[q2], f)) {
              members.push_back(q2);
              consumed[q2] = 1;
            }
          if (members.size() == 1) {
            o << pre << "{\n        const int ti = " << (tany ? te.str() : std::string("0")) << ";\n        (void)ti;\n";
            for (int j = 0; j < 16; j++) {
              if (!((f.jmask >> j) & 1)) continue;
              const int r = (int)((f.rpart >> (4 * j)) & 15);
              for (const std::string& a : arrs)
                o << "        " << a << "[" << j << "] = sv::tmul(" << CF << "[" << f.coef << " + (" << r << " | ti)], "
                  << a << "[" << j << "]);\n";
            }
            o << "      }\n";
            break;
          }
          std::vector<int> rs;  // distinct register parts of the table index
          for (int j = 0; j < 16; j++) {
            const int r = (int)((f.rpart >> (4 * j)) & 15);
            if (((f.jmask >> j) & 1) && std::find(rs.begin(), rs.end(), r) == rs.end()) rs.push_back(r);
          }
          o << "      {  // " << members.size() << " diagonals of one register shape\n";
          for (size_t k = 0; k < rs.size(); k++) o << "        T fr" << k << "{1, 0};\n";
          for (int mq : members) {
            const FOp& g = p.ops[mq];
            const std::string gc = cond_of(g), gi = index_of(g);
            o << "        " << (gc.empty() ? std::string() : "if (" + gc + ") ") << "{\n          const int ti = "
              << (gi.empty() ? std::string("0") : gi) << ";\n          (void)ti;\n";
            for (size_t k = 0; k < rs.size(); k++)
              o << "          fr" << k << " = sv::tmul(" << CF << "[" << g.coef << " + (" << rs[k] << " | ti)], fr" << k
                << ");\n";
            o << "        }\n";
          }
          for (int j = 0; j < 16; j++) {
            if (!((f.jmask >> j) & 1)) continue;
            const int r = (int)((f.rpart >> (4 * j)) & 15);
            const size_t k = std::find(rs.begin(), rs.end(), r) - rs.begin();
            for (const std::string& a : arrs) o << "        " << a << "[" << j << "] = sv::tmul(fr" << k << ", " << a << "[" << j << "]);\n";
          }
          o << "      }\n";
          break;
        }
        case FOP_GRADX:
        case FOP_GRADY:
          if (!adj) return std::string();
          grad_sum(f, "sv::grad_pairs<T, " + std::to_string((int)f.u0) + ", " + (f.type == FOP_GRADX ? "1" : "2") +
                          ">(v, w)");
          break;
        case FOP_GRADZ: {  // invariant under the pending sign flips (both states carry them)
          if (!adj) return std::string();
          unsigned bits = 0;
          for (int j = 0; j < 16; j++) bits |= (unsigned)((f.rpart >> (4 * j)) & 1) << j;
          std::string tbit = "0";
          if (f.tb[0] >= 0) tbit = "((lbase >> " + std::to_string((int)f.tb[0]) + ") & 1)";
          else if (f.ob[0] >= 0) tbit = "(int)((base >> " + std::to_string((int)f.ob[0]) + ") & 1)";
          grad_sum(f, "sv::grad_z<T>(v, w, " + std::to_string(bits) + "u, " + tbit + ")");
          break;
        }
        default:
          return std::string();  // anything else: not specialisable
      }
    }
    flush();
    for (int j = 0; j < 16; j++) o << "      tp[" << P.soff[j] << "] = v[" << j << "];\n";
    if (adj)
      for (int j = 0; j < 16; j++) o << "      tq[" << P.soff[j] << "] = w[" << j << "];\n";
    o << "      __syncthreads();\n    }\n";
  }
  if (adj) {
    o << "    T* const sp = psis[circ];\n"
      << "    T* const sl = lams[circ];\n"
      << "#pragma unroll\n"
      << "    for (int k = 0; k < 16; k++) {\n"
      << "      sv::stg_stream(sp + (base | dtid | DEPK[k]), tile[stid + POSK[k]]);\n"
      << "      sv::stg_stream(sl + (base | dtid | DEPK[k]), ltile[stid + POSK[k]]);\n"
      << "    }\n"
      << "    __syncthreads();  // these buffers are refilled by the prefetch two tiles later\n"
      << "    add_tile();\n"
      << "  }\n"
      << "  if (cur_circ >= 0) flush_grads(cur_circ);\n}\n";
    return o.str();
  }
  o << "#pragma unroll\n"
    << "    for (int k = 0; k < 16; k++) sv::stg_stream(" << (batched ? "st" : "state")
    << " + (base | dtid | DEPK[k]), tile[stid + POSK[k]]);\n"
    << "    __syncthreads();  // this buffer is refilled by the prefetch two tiles later\n"
    << "  }\n}\n";
  return o.str();
}

// ---------------------------------------------------------------- kernel cache
struct CompiledKernel {
  cudaLibrary_t lib = nullptr;
  cudaKernel_t kernel = nullptr;
};

std::mutex g_cache_mutex;
std::unordered_map<std::string, CompiledKernel>& cache() {
  static std::unordered_map<std::string, CompiledKernel> c;
  return c;
}

// ------------------------------------------------------------ on-disk cache
// Compiled cubins are kept across processes in $QIBOJIT_GB300_CACHE (empty or "0":
// off), else $XDG_CACHE_HOME/qibojit_gb300 or ~/.cache/qibojit_gb300.  A file holds
// the full text it was compiled from (options, NVRTC version, header and kernel
// source) and the cubin; it is used only when that text matches exactly and the cubin
// is an ELF image.  Files are written to a temporary name and renamed into place, and
// every disk error just means compiling again.
const char* kCompileOpts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "--diag-suppress=177"};
constexpr int kNumCompileOpts = 3;

std::string disk_cache_dir() {
  const char* e = getenv("QIBOJIT_GB300_CACHE");
  if (e) return (!*e || strcmp(e, "0") == 0) ? std::string() : std::string(e);
  const char* x = getenv("XDG_CACHE_HOME");
  if (x && *x) return std::string(x) + "/qibojit_gb300";
  const char* h = getenv("HOME");
  if (h && *h) return std::string(h) + "/.cache/qibojit_gb300";
  return std::string();
}

uint64_t fnv1a64(const std::string& s) {
  uint64_t h = 1469598103934665603ull;
  for (unsigned char c : s) {
    h ^= c;
    h *= 1099511628211ull;
  }
  return h;
}

bool make_dirs(const std::string& dir) {
  for (size_t i = 1; i <= dir.size(); i++) {
    if (i < dir.size() && dir[i] != '/') continue;
    const std::string part = dir.substr(0, i);
    if (mkdir(part.c_str(), 0755) != 0 && errno != EEXIST) return false;
  }
  return true;
}

const char kCacheMagic[8] = {'S', 'V', 'C', 'U', 'B', 'I', 'N', '1'};

bool disk_load(const std::string& path, const std::string& key, std::vector<char>* cubin) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return false;
  bool ok = false;
  char magic[8];
  uint64_t klen = 0, clen = 0;
  if (fread(magic, 1, 8, f) == 8 && memcmp(magic, kCacheMagic, 8) == 0 && fread(&klen, 8, 1, f) == 1 &&
      klen == key.size()) {
    std::string k(klen, '\0');
    if (fread(&k[0], 1, klen, f) == klen && k == key && fread(&clen, 8, 1, f) == 1 && clen >= 4 &&
        clen < (1ull << 31)) {
      cubin->resize(clen);
      ok = fread(cubin->data(), 1, clen, f) == clen && memcmp(cubin->data(), "\x7f" "ELF", 4) == 0;
    }
  }
  fclose(f);
  if (!ok) cubin->clear();
  return ok;
}

void disk_store(const std::string& dir, const std::string& path, const std::string& key,
                const std::vector<char>& cubin) {
  if (!make_dirs(dir)) return;
  const std::string tmp = path + ".tmp." + std::to_string((long long)getpid()) + "." +
                          std::to_string((unsigned long long)std::hash<std::thread::id>()(std::this_thread::get_id()));
  FILE* f = fopen(tmp.c_str(), "wb");
  if (!f) return;
  const uint64_t klen = key.size(), clen = cubin.size();
  bool ok = fwrite(kCacheMagic, 1, 8, f) == 8 && fwrite(&klen, 8, 1, f) == 1 &&
            fwrite(key.data(), 1, klen, f) == klen && fwrite(&clen, 8, 1, f) == 1 &&
            fwrite(cubin.data(), 1, clen, f) == clen;
  ok = (fclose(f) == 0) && ok;
  if (!ok || rename(tmp.c_str(), path.c_str()) != 0) unlink(tmp.c_str());
}

// NVRTC: source -> cubin for sm_103a (through the on-disk cache)
int compile_cubin(const std::string& body, std::vector<char>* cubin, std::string* log) {
  const Nvrtc& api = nvrtc();
  const std::string src = std::string(kDeviceHeaderText) + "\n" + body;
  const std::string dir = disk_cache_dir();
  std::string key, path;
  if (!dir.empty()) {
    int major = 0, minor = 0;
    if (api.version) api.version(&major, &minor);
    key = "nvrtc " + std::to_string(major) + "." + std::to_string(minor);
    for (int i = 0; i < kNumCompileOpts; i++) key += std::string(" ") + kCompileOpts[i];
    key += "\n" + src;
    char name[64];
    snprintf(name, sizeof(name), "/%016llx_%zu.cubin", (unsigned long long)fnv1a64(key), key.size());
    path = dir + name;
    if (disk_load(path, key, cubin)) return SV_OK;
  }
  nvrtcProgram_t prog = nullptr;
  if (api.create(&prog, src.c_str(), "sv_pass.cu", 0, nullptr, nullptr) != 0) {
    *log = "nvrtcCreateProgram failed";
    return SV_ERR_CUDA;
  }
  const int rc = api.compile(prog, kNumCompileOpts, kCompileOpts);
  size_t n = 0;
  api.log_size(prog, &n);
  log->assign(n, '\0');
  if (n) api.log(prog, &(*log)[0]);
  if (rc == 0) {
    size_t cs = 0;
    api.cubin_size(prog, &cs);
    cubin->resize(cs);
    api.cubin(prog, cubin->data());
  }
  api.destroy(&prog);
  if (rc == 0 && !path.empty()) disk_store(dir, path, key, *cubin);
  return rc == 0 ? SV_OK : SV_ERR_CUDA;
}

}  // namespace

struct PassKernel {
  cudaKernel_t kernel = nullptr;
  int threads = 0, per_sm = 0;
  size_t smem = 0;
};

struct Specialized {
  std::vector<PassKernel> passes;  // indexed like the program's pass blocks
  bool dw = false;                 // compiled for double-word complex128 (cw)
};

bool specialized_is_dw(const Specialized* s) { return s && s->dw; }

void specialized_free(Specialized* s) { delete s; }

// generates, compiles (in parallel, through the process cache) and loads the pass
// kernels of a program: single-state, batched or adjoint (PassMode)
template <typename T>
static int build_kernels(Context* ctx, const sv_program* prog, int mode, std::unique_ptr<Specialized>* out) {
  const int np = prog->npasses;
  const char* name = mode == PASS_ADJOINT ? "sv_apass" : mode == PASS_BATCHED ? "sv_bpass" : "sv_pass";
  auto block = [&](int i) -> const PassParams<T>& {
    return *reinterpret_cast<const PassParams<T>*>(prog->passes.data() + (size_t)i * prog->pass_bytes);
  };
  std::vector<std::string> sources(np);
  for (int i = 0; i < np; i++) {
    sources[i] = pass_source<T>(block(i), name, mode);
    if (sources[i].empty()) return set_error(SV_ERR_UNSUPPORTED, "pass %d holds ops that cannot be specialised", i);
  }
  // compile the sources not in the cache, in parallel
  std::vector<int> todo;
  {
    std::lock_guard<std::mutex> g(g_cache_mutex);
    for (int i = 0; i < np; i++) {
      if (cache().count(sources[i])) continue;
      bool dup = false;
      for (int j : todo) dup |= sources[j] == sources[i];
      if (!dup) todo.push_back(i);
    }
  }
  std::vector<std::vector<char>> cubins(todo.size());
  std::vector<std::string> logs(todo.size());
  std::vector<int> rcs(todo.size(), SV_OK);
  {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t nthr = std::min<size_t>(todo.size(), hw);
    std::vector<std::thread> pool;
    std::mutex m;
    size_t next = 0;
    for (size_t w = 0; w < nthr; w++)
      pool.emplace_back([&] {
        for (;;) {
          size_t k;
          {
            std::lock_guard<std::mutex> g(m);
            if (next >= todo.size()) return;
            k = next++;
          }
          rcs[k] = compile_cubin(sources[todo[k]], &cubins[k], &logs[k]);
        }
      });
    for (auto& th : pool) th.join();
  }
  for (size_t k = 0; k < todo.size(); k++)
    if (rcs[k] != SV_OK)
      return set_error(SV_ERR_CUDA, "runtime compilation of pass %d failed: %.400s", todo[k], logs[k].c_str());
  SV_TRY(check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice"));
  {
    std::lock_guard<std::mutex> g(g_cache_mutex);
    for (size_t k = 0; k < todo.size(); k++) {
      CompiledKernel ck;
      SV_TRY(check_cuda(cudaLibraryLoadData(&ck.lib, cubins[k].data(), nullptr, nullptr, 0, nullptr, nullptr, 0),
                        "cudaLibraryLoadData"));
      SV_TRY(check_cuda(cudaLibraryGetKernel(&ck.kernel, ck.lib, name), "cudaLibraryGetKernel"));
      cache()[sources[todo[k]]] = ck;
    }
  }
  std::unique_ptr<Specialized> s(new Specialized());
  s->passes.resize(np);
  for (int i = 0; i < np; i++) {
    const KernelShape ks = shape_of<T>(prog->kt, mode, mode == PASS_ADJOINT ? adjoint_slots(block(i)) : 0);
    PassKernel& pk = s->passes[i];
    {
      std::lock_guard<std::mutex> g(g_cache_mutex);
      pk.kernel = cache()[sources[i]].kernel;
    }
    pk.threads = ks.threads;
    pk.smem = ks.smem;
    SV_TRY(check_cuda(cudaKernelSetAttributeForDevice(pk.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                      (int)pk.smem, ctx->device),
                      "specialised pass smem attribute"));
    SV_TRY(check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pk.per_sm, (const void*)pk.kernel, pk.threads,
                                                                    pk.smem),
                      "specialised pass occupancy"));
    if (pk.per_sm < 1) return set_error(SV_ERR_ARG, "specialised pass %d does not fit on an SM", i);
  }
  *out = std::move(s);
  return SV_OK;
}

template <typename T>
static int specialize_typed(Context* ctx, sv_program* prog) {
  if (!nvrtc().ok)
    return set_error(SV_ERR_UNSUPPORTED, "the CUDA runtime compiler (libnvrtc.so.13) could not be loaded");
  // specialised passes run the phase-folded plan fastest (no op decoding to pay for)
  SV_TRY(refold_program(prog));
  std::unique_ptr<Specialized> s;
  if (std::is_same<T, c128>::value && !ctx->c128_fp64) {  // complex128 in double-word arithmetic
    SV_TRY(build_kernels<cw>(ctx, prog, PASS_SINGLE, &s));
    s->dw = true;
  } else {
    SV_TRY(build_kernels<T>(ctx, prog, PASS_SINGLE, &s));
  }
  if (prog->spec) specialized_free(prog->spec);
  prog->spec = s.release();
  return SV_OK;
}

int specialize_batched(Context* ctx, sv_program* prog, bool dw) {
  if (!nvrtc().ok)
    return set_error(SV_ERR_UNSUPPORTED, "the CUDA runtime compiler (libnvrtc.so.13) could not be loaded");
  // batched programs keep the unfolded plan: every circuit's coefficients are its own
  // gates' entries, gathered through the plan's coefficient-source map
  if (prog->fold_diagonals) return set_error(SV_ERR_ARG, "batched passes need an unfolded program");
  std::unique_ptr<Specialized> s;
  if (prog->dtype == SV_C128 && dw) {
    SV_TRY(build_kernels<cw>(ctx, prog, PASS_BATCHED, &s));
    s->dw = true;
  } else {
    SV_TRY(prog->dtype == SV_C128 ? build_kernels<c128>(ctx, prog, PASS_BATCHED, &s)
                                   : build_kernels<c64>(ctx, prog, PASS_BATCHED, &s));
  }
  if (prog->bspec) specialized_free(prog->bspec);
  prog->bspec = s.release();
  return SV_OK;
}

int specialized_launch_batched(Context* ctx, const sv_program* prog, int pass, cudaStream_t stream, void* states,
                               const void* coef, int64_t coef_stride, int ncirc) {
  const PassKernel& pk = prog->bspec->passes[pass];
  const int64_t items = ((int64_t)1 << (prog->nqubits - prog->kt)) * ncirc;
  int64_t grid = (int64_t)pk.per_sm * ctx->num_sms;
  if (grid > items) grid = items;
  long long stride = (long long)coef_stride;
  void* args[] = {&states, const_cast<void**>(&coef), &stride, &ncirc};
  SV_TRY(check_cuda(cudaLaunchKernel((const void*)pk.kernel, dim3((unsigned)grid), dim3(pk.threads), args, pk.smem,
                                     stream),
                    "specialised batched pass launch"));
  return SV_OK;
}

int specialize_adjoint(Context* ctx, sv_program* prog) {
  if (!nvrtc().ok)
    return set_error(SV_ERR_UNSUPPORTED, "the CUDA runtime compiler (libnvrtc.so.13) could not be loaded");
  if (prog->fold_diagonals) return set_error(SV_ERR_ARG, "adjoint passes need an unfolded program");
  std::unique_ptr<Specialized> s;
  SV_TRY(prog->dtype == SV_C128 ? build_kernels<c128>(ctx, prog, PASS_ADJOINT, &s)
                                : build_kernels<c64>(ctx, prog, PASS_ADJOINT, &s));
  if (prog->aspec) specialized_free(prog->aspec);
  prog->aspec = s.release();
  return SV_OK;
}

int specialized_launch_adjoint(Context* ctx, const sv_program* prog, int pass, void* psis, void* lams,
                               const void* coef, int64_t coef_stride, int ncirc, double* gpart, int nparams,
                               int gstride) {
  const PassKernel& pk = prog->aspec->passes[pass];
  const int64_t items = ((int64_t)1 << (prog->nqubits - prog->kt)) * ncirc;
  int64_t grid = (int64_t)pk.per_sm * ctx->num_sms;
  if (grid > items) grid = items;
  if (grid > gstride) grid = gstride;  // one gradient column per block
  long long stride = (long long)coef_stride;
  void* args[] = {&psis, &lams, const_cast<void**>(&coef), &stride, &ncirc, &gpart, &nparams, &gstride};
  SV_TRY(check_cuda(cudaLaunchKernel((const void*)pk.kernel, dim3((unsigned)grid), dim3(pk.threads), args, pk.smem,
                                     ctx->stream),
                    "specialised adjoint pass launch"));
  return SV_OK;
}

int specialized_launch(Context* ctx, const sv_program* prog, int pass, void* state) {
  const PassKernel& pk = prog->spec->passes[pass];
  const bool dw = prog->spec->dw;
  const unsigned char* block = (dw ? prog->passes_dw : prog->passes).data() + (size_t)pass * prog->pass_bytes;
  const void* coef = dw ? (const void*)reinterpret_cast<const PassParams<cw>*>(block)->coef
                        : prog->dtype == SV_C128 ? (const void*)reinterpret_cast<const PassParams<c128>*>(block)->coef
                                                 : (const void*)reinterpret_cast<const PassParams<c64>*>(block)->coef;
  const int64_t ntiles = (int64_t)1 << (prog->nqubits - prog->kt);
  int64_t grid = (int64_t)pk.per_sm * ctx->num_sms;
  if (grid > ntiles) grid = ntiles;
  void* args[] = {&state, const_cast<void*>(coef)};
  SV_TRY(check_cuda(cudaLaunchKernel((const void*)pk.kernel, dim3((unsigned)grid), dim3(pk.threads), args, pk.smem,
                                     ctx->stream),
                    "specialised pass launch"));
  return SV_OK;
}

}  // namespace sv

extern "C" {

int sv_program_specialize(sv_context* ctx, sv_program* prog) {
  if (!ctx || !prog) return sv::set_error(SV_ERR_ARG, "null context or program");
  return prog->dtype == SV_C128 ? sv::specialize_typed<sv::c128>(ctx, prog)
                                : sv::specialize_typed<sv::c64>(ctx, prog);
}

}  // extern "C"
