/* Launches the REFERENCE's own kernels (compiled from its headers by ref_kernels.cu into
 * oracle/_ref/ref_kernels_<part>.cubin) on the GPU, for parity tests and for the reference-kernel timings of the
 * benchmark.  Test infrastructure only; the product never links it.
 *
 * The cubins hold device code only, so the reference's host launchers do not exist here; each
 * ref_* function below restates one launcher's launch configuration (grid, block, which
 * template instantiation, the separate reduction launch) with the reference file:lines it
 * follows.  Differences, all outside the kernels: the caller passes the partial-sum buffer (the
 * launchers cudaMalloc a static one, e.g. tsmttsm/genv5.cuh:101-102), launches go to the stream
 * given (the launchers use the legacy default stream), and SPECSMALL's reduction, commented out
 * in its launcher (specsmall.cuh:122-123), is launched, so that SPECSMALL yields a final C as
 * the reference's numeric test expects (numeric_tests.cu:58-64).
 *
 * Kernels are found by their demangled names ("GENV5::blockProductKernel<double, 8, 8, 256,
 * false>"); the CUDA driver is opened with dlopen so the library also loads where no driver is
 * installed (then ref_init fails cleanly).
 *
 * Return values of the launch functions: 1 launched, 0 the reference launcher would return false
 * (shape outside its limits) or the instantiation was not compiled, -1 error (ref_last_error()).
 */
#include <cuda.h>
#include <cxxabi.h>
#include <dirent.h>
#include <dlfcn.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace {

struct Driver {
  CUresult (*Init)(unsigned);
  CUresult (*CtxGetCurrent)(CUcontext*);
  CUresult (*CtxSetCurrent)(CUcontext);
  CUresult (*DeviceGet)(CUdevice*, int);
  CUresult (*DevicePrimaryCtxRetain)(CUcontext*, CUdevice);
  CUresult (*ModuleLoad)(CUmodule*, const char*);
  CUresult (*ModuleGetFunctionCount)(unsigned*, CUmodule);
  CUresult (*ModuleEnumerateFunctions)(CUfunction*, unsigned, CUmodule);
  CUresult (*FuncGetName)(const char**, CUfunction);
  CUresult (*LaunchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                           unsigned, CUstream, void**, void**);
  CUresult (*GetErrorString)(CUresult, const char**);
};

Driver g_drv;
bool g_ready = false;
std::mutex g_mu;
std::map<std::string, CUfunction> g_fn;
std::vector<std::string> g_names;
thread_local std::string g_err;

int fail(const std::string& msg) {
  g_err = msg;
  return -1;
}

bool ok(CUresult r, const char* what) {
  if (r == CUDA_SUCCESS) return true;
  const char* s = nullptr;
  if (g_drv.GetErrorString) g_drv.GetErrorString(r, &s);
  g_err = std::string(what) + ": " + (s ? s : "CUDA error ") + " (" + std::to_string((int)r) + ")";
  return false;
}

template <typename F>
bool sym(void* h, const char* name, F& f) {
  f = reinterpret_cast<F>(dlsym(h, name));
  if (!f) g_err = std::string("libcuda lacks ") + name;
  return f != nullptr;
}

// "void NS::kernel<args>(params)" -> "NS::kernel<args>"
std::string key_of(const char* mangled) {
  const char* z = strstr(mangled, "_Z");
  if (!z) return mangled;
  int st = 0;
  char* d = abi::__cxa_demangle(z, nullptr, nullptr, &st);
  if (!d || st != 0) {
    free(d);
    return mangled;
  }
  std::string s(d);
  free(d);
  if (s.rfind("void ", 0) == 0) s = s.substr(5);
  int depth = 0;
  for (size_t i = 0; i < s.size(); ++i) {
    if (s[i] == '<') ++depth;
    if (s[i] == '>') --depth;
    if (s[i] == '(' && depth == 0) return s.substr(0, i);
  }
  return s;
}

CUfunction find(const std::string& key) {
  auto it = g_fn.find(key);
  return it == g_fn.end() ? nullptr : it->second;
}

// Scalar storage for one kernel argument of the working type.
struct Scalar {
  alignas(16) unsigned char b[16];
};

Scalar scalar(int dt, double re, double im) {
  Scalar s;
  memset(s.b, 0, sizeof s.b);
  if (dt == 0) {
    float f = (float)re;
    memcpy(s.b, &f, 4);
  } else if (dt == 1) {
    memcpy(s.b, &re, 8);
  } else {
    memcpy(s.b, &re, 8);
    memcpy(s.b + 8, &im, 8);
  }
  return s;
}

const char* tname(int dt) {
  switch (dt) {
    case 0: return "float";
    case 1: return "double";
    case 3: return "double2";  // cuDoubleComplex is a typedef of double2
    default: return "?";
  }
}

size_t tsize(int dt) { return dt == 0 ? 4 : dt == 1 ? 8 : 16; }

std::string targs(std::initializer_list<std::string> a) {
  std::string s = "<";
  bool first = true;
  for (auto& x : a) {
    if (!first) s += ", ";
    s += x;
    first = false;
  }
  return s + ">";
}

std::string I(long long v) { return std::to_string(v); }
std::string B(bool v) { return v ? "true" : "false"; }

int launch(CUfunction f, unsigned grid, unsigned bx, unsigned by, void** args, uintptr_t stream) {
  if (!ok(g_drv.LaunchKernel(f, grid, 1, 1, bx, by, 1, 0, (CUstream)stream, args, nullptr),
          "cuLaunchKernel"))
    return -1;
  return 1;
}

}  // namespace

extern "C" {

const char* ref_last_error(void) { return g_err.c_str(); }

/* Opens the driver, makes device 0's primary context current (the one the CUDA runtime and
 * PyTorch use), loads every *.cubin in `dir`.  Returns the number of kernels found, or -1. */
int ref_init(const char* dir) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_ready) return (int)g_fn.size();
  void* h = dlopen("libcuda.so.1", RTLD_NOW | RTLD_GLOBAL);
  if (!h) return fail("cannot open libcuda.so.1 (no NVIDIA driver)");
  if (!(sym(h, "cuInit", g_drv.Init) && sym(h, "cuCtxGetCurrent", g_drv.CtxGetCurrent) &&
        sym(h, "cuCtxSetCurrent", g_drv.CtxSetCurrent) && sym(h, "cuDeviceGet", g_drv.DeviceGet) &&
        sym(h, "cuDevicePrimaryCtxRetain", g_drv.DevicePrimaryCtxRetain) &&
        sym(h, "cuModuleLoad", g_drv.ModuleLoad) &&
        sym(h, "cuModuleGetFunctionCount", g_drv.ModuleGetFunctionCount) &&
        sym(h, "cuModuleEnumerateFunctions", g_drv.ModuleEnumerateFunctions) &&
        sym(h, "cuFuncGetName", g_drv.FuncGetName) && sym(h, "cuLaunchKernel", g_drv.LaunchKernel) &&
        sym(h, "cuGetErrorString", g_drv.GetErrorString)))
    return -1;
  if (!ok(g_drv.Init(0), "cuInit")) return -1;
  CUcontext ctx = nullptr;
  if (!ok(g_drv.CtxGetCurrent(&ctx), "cuCtxGetCurrent")) return -1;
  if (!ctx) {
    CUdevice dev;
    if (!ok(g_drv.DeviceGet(&dev, 0), "cuDeviceGet")) return -1;
    if (!ok(g_drv.DevicePrimaryCtxRetain(&ctx, dev), "cuDevicePrimaryCtxRetain")) return -1;
    if (!ok(g_drv.CtxSetCurrent(ctx), "cuCtxSetCurrent")) return -1;
  }
  DIR* d = opendir(dir);
  if (!d) return fail(std::string("no directory ") + dir);
  std::vector<std::string> files;
  while (dirent* e = readdir(d)) {
    std::string n = e->d_name;
    if (n.size() > 6 && n.compare(n.size() - 6, 6, ".cubin") == 0) files.push_back(std::string(dir) + "/" + n);
  }
  closedir(d);
  if (files.empty()) return fail(std::string("no .cubin files in ") + dir);
  for (auto& f : files) {
    CUmodule m;
    if (!ok(g_drv.ModuleLoad(&m, f.c_str()), ("cuModuleLoad " + f).c_str())) return -1;
    unsigned cnt = 0;
    if (!ok(g_drv.ModuleGetFunctionCount(&cnt, m), "cuModuleGetFunctionCount")) return -1;
    std::vector<CUfunction> fs(cnt);
    if (cnt && !ok(g_drv.ModuleEnumerateFunctions(fs.data(), cnt, m), "cuModuleEnumerateFunctions"))
      return -1;
    for (CUfunction fn : fs) {
      const char* nm = nullptr;
      if (!ok(g_drv.FuncGetName(&nm, fn), "cuFuncGetName")) return -1;
      std::string k = key_of(nm);
      g_fn[k] = fn;
      g_names.push_back(k);
    }
  }
  g_ready = true;
  return (int)g_fn.size();
}

int ref_kernel_count(void) { return (int)g_names.size(); }
const char* ref_kernel_name(int i) {
  return (i >= 0 && i < (int)g_names.size()) ? g_names[i].c_str() : "";
}

/* Bytes of the partial-sum buffer a TSMTTSM variant needs (its blockResults layout):
 * GENV5 / GENV3X / SPECSMALL blockCount*N*ldc accumulators (genv5.cuh:20, genv3x.cuh:20,
 * specsmall.cuh:21); SPECSMALL with PseudoQuad 16 bytes each. */
size_t ref_tsmttsm_temp_bytes(const char* variant, int dtype, int M, int N, int ldc, int blockCount) {
  std::string v = variant;
  size_t acc = v == "SPECSMALL_PQ" ? 16 : tsize(dtype);
  size_t cells = (size_t)N * ldc;
  return (size_t)blockCount * cells * acc;
}

/* TSMTTSM C = alpha A^T B + beta C with one of the reference's kernels.
 * variant: "GENV5" (genv5.cuh:93-114), "GENV3X" (genv3x.cuh:83-106, THREAD_PER_N = 2),
 * "SPECSMALL" / "SPECSMALL_PQ" (specsmall.cuh:94-125 with iT = T / PseudoQuad, then its
 * deviceReduce, specsmall.cuh:10-26).  dtype 0 float, 1 double.  GENV6 (genv6.cuh:67-89) is not
 * offered: its kernel reads past a shared array (genv6.cuh:54) and faulted on GB300. */
int ref_tsmttsm(const char* variant, int dtype, int M, int N, int K, uintptr_t A, int lda, double alpha,
                uintptr_t Bp, int ldb, double beta, uintptr_t C, int ldc, int blockCount, uintptr_t temp,
                size_t temp_bytes, uintptr_t stream) {
  if (!g_ready) return fail("ref_init has not succeeded");
  std::string v = variant;
  if (dtype != 0 && dtype != 1) return 0;
  if (blockCount < 1) return fail("blockCount < 1");
  // The launchers' own limits: (M, N) <= 32 (genv5.cuh:99, specsmall.cuh:99) and the static
  // buffer's 100*100*1000 accumulators (genv5.cuh:103, genv3x.cuh:95, specsmall.cuh:102).
  if ((long long)blockCount * M * N > 100LL * 100 * 1000) return 0;
  if ((v == "GENV5" || v == "SPECSMALL" || v == "SPECSMALL_PQ") && (M > 32 || N > 32)) return 0;
  if (temp_bytes < ref_tsmttsm_temp_bytes(variant, dtype, M, N, ldc, blockCount))
    return fail("partial-sum buffer too small");
  const std::string T = tname(dtype);
  Scalar al = scalar(dtype, alpha, 0), be = scalar(dtype, beta, 0);
  void* tmp = (void*)temp;
  const bool tr = N > M;
  // Kernel arguments of blockProductKernel: (A, B, out, K, lda, ldb, ldc), operands swapped for
  // the transposed form (genv5.cuh:106-112).
  uintptr_t a0 = tr ? Bp : A, b0 = tr ? A : Bp;
  int la = tr ? ldb : lda, lb = tr ? lda : ldb;
  int KM = tr ? N : M, KN = tr ? M : N;
  void* pargs[] = {&a0, &b0, &tmp, &K, &la, &lb, &ldc};
  unsigned rgrid = (unsigned)(M * N / 256 + 1);  // M * N / 256 + 1 blocks of 256 (genv5.cuh:111)
  if (v == "GENV5" || v == "GENV3X") {
    std::string k = v + "::blockProductKernel" +
                    (v == "GENV5" ? targs({T, I(KM), I(KN), "256", B(tr)})
                                  : targs({T, I(KM), I(KN), "256", B(tr), "2"}));
    CUfunction f = find(k), r = find(v + "::deviceReduce" + targs({T, I(M), I(N)}));
    if (!f || !r) return 0;
    if (launch(f, blockCount, 256, 1, pargs, stream) != 1) return -1;
    if (v == "GENV5") {
      // GENV5's reduction takes size_t leading dimensions (genv5.cuh:10-12).
      size_t la64 = lda, lb64 = ldb, lc64 = ldc;
      void* rargs[] = {&tmp, &C, al.b, be.b, &blockCount, &la64, &lb64, &lc64};
      return launch(r, rgrid, 256, 1, rargs, stream);
    }
    void* rargs[] = {&tmp, &C, al.b, be.b, &blockCount, &lda, &ldb, &ldc};
    return launch(r, rgrid, 256, 1, rargs, stream);
  }
  if (v == "SPECSMALL" || v == "SPECSMALL_PQ") {
    if (v == "SPECSMALL_PQ" && dtype != 1) return 0;
    const std::string iT = v == "SPECSMALL_PQ" ? "PseudoQuad" : T;
    const bool self = !tr && M == N && A == Bp;  // specsmall.cuh:112
    CUfunction f = find("SPECSMALL::blockProductKernel" + targs({T, iT, I(KM), I(KN), "256", B(tr), B(self)}));
    CUfunction r = find("SPECSMALL::deviceReduce" + targs({T, iT, I(M), I(N)}));
    if (!f || !r) return 0;
    if (launch(f, blockCount, 256, 1, pargs, stream) != 1) return -1;
    void* rargs[] = {&tmp, &C, al.b, be.b, &blockCount, &lda, &ldb, &ldc};
    return launch(r, rgrid, 256, 1, rargs, stream);
  }
  return fail("unknown TSMTTSM variant " + v);
}

/* TSMM C = alpha A B + beta C with one of the reference's kernels.
 * variant: "FIX3" (tsmm/fix3.cuh:41-65; in place when A == C), "FIX_FB" (fix_fb.cuh:72-102;
 * refuses A == C), "FIX_IP_GHOST" (fix_ip_ghost.cuh:24-44; in place only, A == C).
 * dtype 0 float, 1 double, 3 complex double (FIX_IP_GHOST only). */
int ref_tsmm(const char* variant, int dtype, int M, int N, int K, uintptr_t A, int lda, double alpha_re,
             double alpha_im, uintptr_t Bp, int ldb, double beta_re, double beta_im, uintptr_t C, int ldc,
             int blockCount, uintptr_t stream) {
  if (!g_ready) return fail("ref_init has not succeeded");
  std::string v = variant;
  const std::string T = tname(dtype);
  if (std::string(T) == "?") return 0;
  Scalar al = scalar(dtype, alpha_re, alpha_im), be = scalar(dtype, beta_re, beta_im);
  const bool beta_zero = beta_re == 0.0 && beta_im == 0.0;  // eq(beta, Tzero), fix3.cuh:57
  if (v == "FIX3" || v == "FIX_FB") {
    if (dtype == 3) return 0;
    if (v == "FIX_FB" && A == C) return 0;  // fix_fb.cuh:74
    if (blockCount < 1) return fail("blockCount < 1");
    int bs = v == "FIX3" ? ((M * N * 8 > 10 * 1024) ? 256 : 128)   // fix3.cuh:47
                         : ((M * N > 1024) ? 1024 : 256);          // fix_fb.cuh:78
    std::string name = (v == "FIX3" ? "tsmm_fix3_kernel" : "tsmm_fix_fb_kernel") +
                       targs({T, I(M), I(N), I(bs), B(beta_zero)});
    CUfunction f = find(name);
    if (!f) return 0;
    void* args[] = {&A, &Bp, &C, &K, &lda, &ldb, &ldc, al.b, be.b};
    return launch(f, blockCount, bs, 1, args, stream);
  }
  if (v == "FIX_IP_GHOST") {
    if (A != C) return 0;  // fix_ip_ghost.cuh:29
    CUfunction f = find("fix_ip_ghost_kernel" + targs({T, I(N), I(M)}));
    if (!f) return 0;
    // block (N, 128 / N), grid K / block.y + 1 (fix_ip_ghost.cuh:31-41); blockCount unused.
    unsigned by = 128 / N;
    unsigned grid = (unsigned)(K / (int)by + 1);
    void* args[] = {&C, &Bp, al.b, be.b, &K, &ldc, &ldb};
    return launch(f, grid, N, by, args, stream);
  }
  return fail("unknown TSMM variant " + v);
}

}  // extern "C"
