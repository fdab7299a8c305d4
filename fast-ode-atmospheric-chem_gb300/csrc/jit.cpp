// The per-mechanism module of the generated variant: the plan's generated
// PTX (codegen.cpp) linked with the relocatable integrator (generated.cu,
// compiled at build time and embedded in this library) by nvJitLink, loaded
// as a CUDA library, kept on disk by content hash.
//
// nvJitLink is opened at run time (dlopen), so the library loads on hosts
// without it; fo_plan_generate then fails with a clear message. Linking runs
// ptxas on the generated code, which takes about a minute for a
// 210-species / 500-reaction mechanism (200,000 multiply-adds of straight-line
// code); the cache makes that a one-time cost per mechanism and host.
#include "jit.h"

#include <cuda_runtime.h>
#include <dlfcn.h>
#include <nvJitLink.h>
#include <sys/stat.h>
#include <unistd.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "codegen.h"

// the relocatable integrator (embed.cpp)
extern "C" const unsigned char fo_generated_rdc_begin[];
extern "C" const unsigned char fo_generated_rdc_end[];

namespace fo {
namespace {

struct JitLink {
  bool loaded = false;
  std::string error;
  decltype(&__nvJitLinkCreate_13_0) create = nullptr;
  decltype(&__nvJitLinkDestroy_13_0) destroy = nullptr;
  decltype(&__nvJitLinkAddData_13_0) add_data = nullptr;
  decltype(&__nvJitLinkComplete_13_0) complete = nullptr;
  decltype(&__nvJitLinkGetLinkedCubinSize_13_0) cubin_size = nullptr;
  decltype(&__nvJitLinkGetLinkedCubin_13_0) cubin = nullptr;
  decltype(&__nvJitLinkGetErrorLogSize_13_0) error_log_size = nullptr;
  decltype(&__nvJitLinkGetErrorLog_13_0) error_log = nullptr;
};

std::mutex g_jit_mutex;

const JitLink& jitlink() {
  static JitLink api;
  static bool tried = false;
  std::lock_guard<std::mutex> lock(g_jit_mutex);
  if (tried) return api;
  tried = true;
  const char* names[] = {"libnvJitLink.so.13", "libnvJitLink.so", "/usr/local/cuda/lib64/libnvJitLink.so.13"};
  void* h = nullptr;
  for (const char* nm : names)
    if ((h = dlopen(nm, RTLD_NOW | RTLD_LOCAL)) != nullptr) break;
  if (!h) {
    api.error = "libnvJitLink.so.13 (CUDA 13 nvJitLink) could not be opened: the generated variant needs it";
    return api;
  }
  bool ok = true;
  auto sym = [&](auto& fn, const char* name) {
    fn = reinterpret_cast<std::remove_reference_t<decltype(fn)>>(dlsym(h, name));
    if (!fn) ok = false;
  };
  sym(api.create, "__nvJitLinkCreate_13_0");
  sym(api.destroy, "__nvJitLinkDestroy_13_0");
  sym(api.add_data, "__nvJitLinkAddData_13_0");
  sym(api.complete, "__nvJitLinkComplete_13_0");
  sym(api.cubin_size, "__nvJitLinkGetLinkedCubinSize_13_0");
  sym(api.cubin, "__nvJitLinkGetLinkedCubin_13_0");
  sym(api.error_log_size, "__nvJitLinkGetErrorLogSize_13_0");
  sym(api.error_log, "__nvJitLinkGetErrorLog_13_0");
  if (!ok) {
    api.error = "libnvJitLink lacks the CUDA 13.0 entry points";
    return api;
  }
  api.loaded = true;
  return api;
}

// The link: sm_103a; at most 128 registers per thread, the integrator
// kernel's budget for sixteen groups per SM, for the generated functions too;
// ptxas optimizes the module's functions (the factorization's pieces among
// them) on all host cores at once.
const char* const kLinkOptions[] = {"-arch=sm_103a", "-O3", "-maxrregcount=128", "-Xptxas=--split-compile=0"};

uint64_t fnv1a(uint64_t h, const void* data, size_t n) {
  const unsigned char* p = static_cast<const unsigned char*>(data);
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}

std::string default_cache_dir() {
  if (const char* e = std::getenv("FASTODE_GB300_CACHE")) return e;
  if (const char* x = std::getenv("XDG_CACHE_HOME")) return std::string(x) + "/fastode_gb300";
  if (const char* h = std::getenv("HOME")) return std::string(h) + "/.cache/fastode_gb300";
  return "";
}

void make_dirs(const std::string& dir) {
  std::string cur;
  std::stringstream ss(dir);
  std::string part;
  if (!dir.empty() && dir[0] == '/') cur = "/";
  while (std::getline(ss, part, '/')) {
    if (part.empty()) continue;
    cur += part + "/";
    mkdir(cur.c_str(), 0755);
  }
}

bool read_file(const std::string& path, std::vector<char>* out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  f.seekg(0, std::ios::end);
  const std::streamoff n = f.tellg();
  if (n <= 0) return false;
  f.seekg(0);
  out->resize((size_t)n);
  f.read(out->data(), n);
  return (bool)f;
}

void write_file_atomic(const std::string& path, const std::vector<char>& data) {
  const std::string tmp = path + ".tmp" + std::to_string(getpid());
  {
    std::ofstream f(tmp, std::ios::binary);
    if (!f) return;
    f.write(data.data(), (std::streamsize)data.size());
    if (!f) {
      std::remove(tmp.c_str());
      return;
    }
  }
  if (std::rename(tmp.c_str(), path.c_str()) != 0) std::remove(tmp.c_str());
}

bool link(const std::string& ptx, std::vector<char>* cubin, std::string* err) {
  const JitLink& api = jitlink();
  if (!api.loaded) {
    *err = api.error;
    return false;
  }
  nvJitLinkHandle h = nullptr;
  if (api.create(&h, (uint32_t)(sizeof(kLinkOptions) / sizeof(kLinkOptions[0])), kLinkOptions) !=
      NVJITLINK_SUCCESS) {
    *err = "nvJitLinkCreate failed";
    return false;
  }
  auto log = [&]() {
    size_t n = 0;
    std::string s;
    if (api.error_log_size(h, &n) == NVJITLINK_SUCCESS && n > 1) {
      s.resize(n);
      api.error_log(h, &s[0]);
      s.resize(n - 1);
    }
    return s;
  };
  bool ok = api.add_data(h, NVJITLINK_INPUT_CUBIN, fo_generated_rdc_begin,
                         (size_t)(fo_generated_rdc_end - fo_generated_rdc_begin), "generated.cu") == NVJITLINK_SUCCESS;
  ok = ok && api.add_data(h, NVJITLINK_INPUT_PTX, ptx.data(), ptx.size(), "mechanism.ptx") == NVJITLINK_SUCCESS;
  ok = ok && api.complete(h) == NVJITLINK_SUCCESS;
  size_t n = 0;
  ok = ok && api.cubin_size(h, &n) == NVJITLINK_SUCCESS && n > 0;
  if (ok) {
    cubin->resize(n);
    ok = api.cubin(h, cubin->data()) == NVJITLINK_SUCCESS;
  }
  if (!ok) *err = "nvJitLink failed: " + log();
  api.destroy(&h);
  return ok;
}

}  // namespace

struct GenModule {
  cudaLibrary_t lib = nullptr;
  cudaKernel_t kernel = nullptr;        // fo_generated_solve_kernel
  cudaKernel_t multi_kernel = nullptr;  // fo_generated_multi_kernel
  cudaKernel_t adjoint_kernel = nullptr;  // fo_generated_adjoint_kernel
  std::mutex mutex;
  int configured_smem[3][64] = {};
};

int gen_create(const std::vector<const HostTables*>& ts, const std::vector<GenOptions>& opts, const char* cache_dir,
               GenModule** out, fo_gen_info* info, std::string* err) {
  const auto t0 = std::chrono::steady_clock::now();
  *out = nullptr;
  std::string ptx;
  try {
    ptx = generate_ptx(ts, opts);
  } catch (const std::exception& e) {
    *err = std::string("code generation failed: ") + e.what();
    return FO_E_INVALID;
  }
  int runtime = 0;
  cudaRuntimeGetVersion(&runtime);
  uint64_t h = 1469598103934665603ull;
  h = fnv1a(h, ptx.data(), ptx.size());
  h = fnv1a(h, fo_generated_rdc_begin, (size_t)(fo_generated_rdc_end - fo_generated_rdc_begin));
  h = fnv1a(h, &runtime, sizeof(runtime));
  for (const char* o : kLinkOptions) h = fnv1a(h, o, std::strlen(o));
  char key[32];
  std::snprintf(key, sizeof(key), "gen-%016llx.cubin", (unsigned long long)h);
  const std::string dir = cache_dir ? std::string(cache_dir) : default_cache_dir();
  const std::string path = dir.empty() ? "" : dir + "/" + key;
  std::vector<char> cubin;
  bool cached = !path.empty() && read_file(path, &cubin);
  if (!cached) {
    if (!link(ptx, &cubin, err)) return FO_E_UNSUPPORTED;
    if (!path.empty()) {
      make_dirs(dir);
      write_file_atomic(path, cubin);
    }
  }
  GenModule* m = new GenModule;
  cudaError_t e = cudaLibraryLoadData(&m->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (e == cudaSuccess) e = cudaLibraryGetKernel(&m->kernel, m->lib, "fo_generated_solve_kernel");
  if (e == cudaSuccess) e = cudaLibraryGetKernel(&m->multi_kernel, m->lib, "fo_generated_multi_kernel");
  if (e == cudaSuccess) e = cudaLibraryGetKernel(&m->adjoint_kernel, m->lib, "fo_generated_adjoint_kernel");
  cudaFuncAttributes attr;
  std::memset(&attr, 0, sizeof(attr));
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&attr, reinterpret_cast<const void*>(m->kernel));
  if (e != cudaSuccess) {
    *err = std::string("loading the generated module: ") + cudaGetErrorString(e);
    if (m->lib) cudaLibraryUnload(m->lib);
    delete m;
    return FO_E_CUDA;
  }
  if (info) {
    std::memset(info, 0, sizeof(*info));
    info->from_cache = cached ? 1 : 0;
    info->registers = attr.numRegs;
    info->tile = opts.empty() ? 0 : opts[0].tile;
    info->local_bytes = (int32_t)attr.localSizeBytes;
    info->ptx_bytes = (int64_t)ptx.size();
    info->cubin_bytes = (int64_t)cubin.size();
    info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  *out = m;
  return FO_OK;
}

int gen_check(const HostTables& t, const GenOptions& opt, bool do_link, fo_gen_info* info, std::string* err) {
  const auto t0 = std::chrono::steady_clock::now();
  std::string ptx;
  try {
    ptx = generate_ptx(t, opt);
  } catch (const std::exception& e) {
    *err = std::string("code generation failed: ") + e.what();
    return FO_E_INVALID;
  }
  std::vector<char> cubin;
  if (do_link && !link(ptx, &cubin, err)) return FO_E_UNSUPPORTED;
  if (info) {
    std::memset(info, 0, sizeof(*info));
    info->tile = opt.tile;
    info->ptx_bytes = (int64_t)ptx.size();
    info->cubin_bytes = (int64_t)cubin.size();
    info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  return FO_OK;
}

void gen_destroy(GenModule* m) {
  if (!m) return;
  if (m->lib) cudaLibraryUnload(m->lib);
  delete m;
}

namespace {

// The dynamic shared-memory limit above 48 KB, set once per kernel, device
// and size under the module's lock.
cudaError_t ensure_smem(GenModule* m, int which, const void* fn, size_t smem) {
  if (smem <= 48 * 1024) return cudaSuccess;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(m->mutex);
  if ((int)smem > m->configured_smem[which][dev]) {
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    m->configured_smem[which][dev] = (int)smem;
  }
  return cudaSuccess;
}

// Whether `grid` one-warp blocks of kernel `fn` with `smem` bytes of dynamic
// shared memory are all resident at once on the current device (what a
// cooperative launch needs).
bool all_resident(const void* fn, int grid, size_t smem) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return false;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 32, smem) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  return (int64_t)per_sm * sms >= grid;
}

}  // namespace

bool gen_resident(GenModule* m, bool multi, int grid, size_t smem) {
  const void* fn = reinterpret_cast<const void*>(multi ? m->multi_kernel : m->kernel);
  if (ensure_smem(m, multi ? 1 : 0, fn, smem) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  return all_resident(fn, grid, smem);
}

cudaError_t gen_launch(GenModule* m, const SolveParams& p, int grid, size_t smem, cudaStream_t stream) {
  const void* fn = reinterpret_cast<const void*>(m->kernel);
  cudaError_t e = ensure_smem(m, 0, fn, smem);
  if (e != cudaSuccess) return e;
  SolveParams q = p;
  void* args[] = {&q};
  // lockstep rounds need every block resident: a cooperative launch; a grid
  // that does not fit runs without rounds
  if (q.rounds != nullptr && all_resident(fn, grid, smem))
    return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(32), args, smem, stream);
  q.rounds = nullptr;
  return cudaLaunchKernel(fn, dim3(grid), dim3(32), args, smem, stream);
}

cudaError_t gen_launch_adjoint(GenModule* m, const AdjParams& a, int grid, size_t smem, cudaStream_t stream) {
  const void* fn = reinterpret_cast<const void*>(m->adjoint_kernel);
  cudaError_t e = ensure_smem(m, 2, fn, smem);
  if (e != cudaSuccess) return e;
  AdjParams q = a;
  void* args[] = {&q};
  return cudaLaunchKernel(fn, dim3(grid), dim3(32), args, smem, stream);
}

cudaError_t gen_launch_multi(GenModule* m, const SolveParams* batches, int nb, const int32_t* starts,
                             int32_t* queue, double* scratch, int64_t slot_doubles, int grid, size_t smem,
                             bool cooperative, cudaStream_t stream) {
  const void* fn = reinterpret_cast<const void*>(m->multi_kernel);
  cudaError_t e = ensure_smem(m, 1, fn, smem);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(queue, 0, sizeof(int32_t), stream);
  if (e != cudaSuccess) return e;
  void* args[] = {&batches, &nb, &starts, &queue, &scratch, &slot_doubles};
  if (cooperative) return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(32), args, smem, stream);
  return cudaLaunchKernel(fn, dim3(grid), dim3(32), args, smem, stream);
}

}  // namespace fo
