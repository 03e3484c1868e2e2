/*
 * C-ABI runtime: run-time compilation of generated stencil modules (NVRTC,
 * sm_103a cubins cached on disk), kernel lookup, and the FDM step loop.
 *
 * Every entry point returns an int status (0 = ok) and never lets a C++
 * exception cross the ABI; prml_last_error() gives the message of the last
 * failure on the calling thread.  See include/pararealml_gb300.h.
 */
#include <cuda.h>
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <nvrtc.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>
#include <mutex>
#include <unistd.h>

#include "prml_internal.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) { return prml_set_error(code, msg); }

std::vector<std::string> split(const char* s, char sep) {
  std::vector<std::string> out;
  if (!s) return out;
  std::string cur;
  for (const char* p = s; *p; ++p) {
    if (*p == sep) {
      if (!cur.empty()) out.push_back(cur);
      cur.clear();
    } else {
      cur.push_back(*p);
    }
  }
  if (!cur.empty()) out.push_back(cur);
  return out;
}

/* Driver API entry points, resolved from libcuda.so.1 on first use so that
 * the library itself loads on machines without a GPU driver. */
struct Driver {
  bool ok = false;
  CUresult (*GetErrorString)(CUresult, const char**) = nullptr;
  CUresult (*CtxGetCurrent)(CUcontext*) = nullptr;
  CUresult (*ModuleLoadData)(CUmodule*, const void*) = nullptr;
  CUresult (*ModuleUnload)(CUmodule) = nullptr;
  CUresult (*ModuleGetFunction)(CUfunction*, CUmodule, const char*) = nullptr;
  CUresult (*FuncSetAttribute)(CUfunction, CUfunction_attribute, int) = nullptr;
  CUresult (*OccupancyMaxActiveBlocksPerMultiprocessor)(int*, CUfunction, int, size_t) = nullptr;
  CUresult (*LaunchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                           unsigned, CUstream, void**, void**) = nullptr;
};

Driver g_drv;
std::mutex g_drv_mu;

template <typename F>
bool bind(void* h, const char* name, F& fn) {
  fn = reinterpret_cast<F>(dlsym(h, name));
  return fn != nullptr;
}

bool driver() {
  std::lock_guard<std::mutex> lock(g_drv_mu);
  if (g_drv.ok) return true;
  void* h = dlopen("libcuda.so.1", RTLD_NOW | RTLD_LOCAL);
  if (!h) return false;
  Driver d;
  d.ok = bind(h, "cuGetErrorString", d.GetErrorString) &&
         bind(h, "cuCtxGetCurrent", d.CtxGetCurrent) &&
         bind(h, "cuModuleLoadData", d.ModuleLoadData) &&
         bind(h, "cuModuleUnload", d.ModuleUnload) &&
         bind(h, "cuModuleGetFunction", d.ModuleGetFunction) &&
         bind(h, "cuFuncSetAttribute", d.FuncSetAttribute) &&
         bind(h, "cuOccupancyMaxActiveBlocksPerMultiprocessor",
              d.OccupancyMaxActiveBlocksPerMultiprocessor) &&
         bind(h, "cuLaunchKernel", d.LaunchKernel);
  if (d.ok) g_drv = d;
  return d.ok;
}

const char* cu_name(CUresult r) {
  const char* s = nullptr;
  if (g_drv.GetErrorString) g_drv.GetErrorString(r, &s);
  return s ? s : "unknown CUDA driver error";
}

#define PRML_CU(call)                                                          \
  do {                                                                         \
    CUresult _r = (call);                                                      \
    if (_r != CUDA_SUCCESS)                                                    \
      return fail(PRML_ERR_CUDA, std::string(#call) + ": " + cu_name(_r));     \
  } while (0)

int ensure_context() {
  /* Attach to the runtime's primary context of the current device (the one
   * PyTorch uses), creating it if this is the first CUDA call. */
  if (!driver()) return fail(PRML_ERR_CUDA, "cannot load the CUDA driver (libcuda.so.1)");
  cudaError_t e = cudaFree(nullptr);
  if (e != cudaSuccess)
    return fail(PRML_ERR_CUDA, std::string("cudaFree(0): ") + cudaGetErrorString(e));
  CUcontext ctx = nullptr;
  PRML_CU(g_drv.CtxGetCurrent(&ctx));
  if (!ctx) return fail(PRML_ERR_CUDA, "no current CUDA context");
  return PRML_OK;
}

bool read_file(const std::string& path, std::string& out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::ostringstream ss;
  ss << f.rdbuf();
  out = ss.str();
  return !out.empty();
}

bool write_file_atomic(const std::string& path, const std::string& data) {
  std::string tmp = path + ".tmp." + std::to_string(getpid());
  {
    std::ofstream f(tmp, std::ios::binary);
    if (!f) return false;
    f.write(data.data(), (std::streamsize)data.size());
    if (!f) return false;
  }
  return std::rename(tmp.c_str(), path.c_str()) == 0;
}

struct Module {
  CUmodule mod = nullptr;
};

struct Kernel {
  CUfunction fn = nullptr;
  int smem = 0;
};

}  // namespace

int prml_set_error(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

extern "C" {

const char* prml_last_error(void) { return g_last_error.c_str(); }

int prml_abi_version(void) { return PRML_ABI_VERSION; }

int prml_step_params_size(void) { return (int)sizeof(prml_step_params); }

int prml_jit_compile(const char* source, const char* include_dirs, const char* arch,
                     const char* extra_options, const char* cache_path, char* log,
                     long long log_len) {
  if (!source || !include_dirs || !arch || !cache_path)
    return fail(PRML_ERR_ARG, "prml_jit_compile: null argument");
  std::string cubin;
  if (read_file(cache_path, cubin)) return PRML_OK;
  nvrtcProgram prog;
  if (nvrtcCreateProgram(&prog, source, "prml_generated.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
    return fail(PRML_ERR_COMPILE, "nvrtcCreateProgram failed");
  std::vector<std::string> opt_store;
  opt_store.push_back(std::string("--gpu-architecture=") + arch);
  for (const std::string& d : split(include_dirs, ';')) opt_store.push_back("--include-path=" + d);
  opt_store.push_back("-std=c++17");
  opt_store.push_back("-lineinfo");
  for (const std::string& o : split(extra_options, ' ')) opt_store.push_back(o);
  std::vector<const char*> opts;
  for (const std::string& o : opt_store) opts.push_back(o.c_str());
  nvrtcResult rc = nvrtcCompileProgram(prog, (int)opts.size(), opts.data());
  size_t nlog = 0;
  nvrtcGetProgramLogSize(prog, &nlog);
  std::string logs(nlog, '\0');
  if (nlog) nvrtcGetProgramLog(prog, &logs[0]);
  if (log && log_len > 0) {
    std::strncpy(log, logs.c_str(), (size_t)log_len - 1);
    log[log_len - 1] = '\0';
  }
  if (rc != NVRTC_SUCCESS) {
    nvrtcDestroyProgram(&prog);
    return fail(PRML_ERR_COMPILE, std::string("NVRTC: ") + nvrtcGetErrorString(rc) + "\n" + logs);
  }
  size_t n = 0;
  nvrtcGetCUBINSize(prog, &n);
  cubin.resize(n);
  nvrtcGetCUBIN(prog, &cubin[0]);
  nvrtcDestroyProgram(&prog);
  if (!write_file_atomic(cache_path, cubin))
    return fail(PRML_ERR_ARG, std::string("cannot write cubin cache ") + cache_path);
  return PRML_OK;
}

int prml_module_load(const char* cubin_path, void** module_out) {
  if (!cubin_path || !module_out) return fail(PRML_ERR_ARG, "prml_module_load: null argument");
  int rc = ensure_context();
  if (rc) return rc;
  std::string cubin;
  if (!read_file(cubin_path, cubin))
    return fail(PRML_ERR_ARG, std::string("cannot read cubin ") + cubin_path);
  Module* m = new Module();
  CUresult r = g_drv.ModuleLoadData(&m->mod, cubin.data());
  if (r != CUDA_SUCCESS) {
    delete m;
    return fail(PRML_ERR_CUDA, std::string("cuModuleLoadData: ") + cu_name(r));
  }
  *module_out = m;
  return PRML_OK;
}

int prml_module_unload(void* module) {
  Module* m = static_cast<Module*>(module);
  if (!m) return PRML_OK;
  if (m->mod) g_drv.ModuleUnload(m->mod);
  delete m;
  return PRML_OK;
}

int prml_module_kernel(void* module, const char* name, int smem_bytes, void** kernel_out) {
  Module* m = static_cast<Module*>(module);
  if (!m || !name || !kernel_out || smem_bytes < 0)
    return fail(PRML_ERR_ARG, "prml_module_kernel: bad argument");
  Kernel* k = new Kernel();
  CUresult r = g_drv.ModuleGetFunction(&k->fn, m->mod, name);
  if (r != CUDA_SUCCESS) {
    delete k;
    return fail(PRML_ERR_ARG, std::string("kernel ") + name + " not found: " + cu_name(r));
  }
  k->smem = smem_bytes;
  if (smem_bytes > 48 * 1024) {
    r = g_drv.FuncSetAttribute(k->fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, smem_bytes);
    if (r != CUDA_SUCCESS) {
      delete k;
      return fail(PRML_ERR_CUDA, std::string("cuFuncSetAttribute(smem): ") + cu_name(r));
    }
  }
  *kernel_out = k;
  return PRML_OK;
}

int prml_kernel_free(void* kernel) {
  delete static_cast<Kernel*>(kernel);
  return PRML_OK;
}

int prml_kernel_occupancy(void* kernel, int block, int* blocks_per_sm) {
  Kernel* k = static_cast<Kernel*>(kernel);
  if (!k || !blocks_per_sm) return fail(PRML_ERR_ARG, "prml_kernel_occupancy: bad argument");
  PRML_CU(g_drv.OccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k->fn, block, k->smem));
  return PRML_OK;
}

static int launch_step(Kernel* k, int block, int gx, int gy, int gz, prml_step_params* p,
                       CUstream stream) {
  void* args[] = {p};
  CUresult r = g_drv.LaunchKernel(k->fn, gx, gy, gz, block, 1, 1, k->smem, stream, args, nullptr);
  if (r != CUDA_SUCCESS) return fail(PRML_ERR_CUDA, std::string("cuLaunchKernel: ") + cu_name(r));
  return PRML_OK;
}

static int check_geometry(const prml_step_params* base, int tile_x, int tile_y, int block) {
  if (!base) return fail(PRML_ERR_ARG, "null params");
  if (base->nx < 1 || base->ny < 1 || base->batch < 1 || base->pitch < base->ny)
    return fail(PRML_ERR_ARG, "bad mesh geometry in params");
  if (tile_x < 1 || tile_y < 1 || block < 32 || block > 1024)
    return fail(PRML_ERR_ARG, "bad tile or block size");
  if (base->batch > 65535) return fail(PRML_ERR_ARG, "batch exceeds 65535 instances");
  long long gy = (base->nx + tile_x - 1) / tile_x;
  if (gy > 65535) return fail(PRML_ERR_ARG, "too many row tiles");
  return PRML_OK;
}

int prml_fdm_run(void* kernel, int block, int tile_x, int tile_y,
                 const prml_step_params* base, const void* y0, long long y0_bstride,
                 void* traj, long long traj_bstride, long long traj_step_stride,
                 void* work_a, void* work_b, long long work_bstride, long long n_steps,
                 int save_every, double t0, double dt, void* stream) {
  Kernel* k = static_cast<Kernel*>(kernel);
  if (!k) return fail(PRML_ERR_ARG, "prml_fdm_run: null kernel");
  int rc = check_geometry(base, tile_x, tile_y, block);
  if (rc) return rc;
  if (!y0 || !traj || n_steps < 0 || save_every < 1)
    return fail(PRML_ERR_ARG, "prml_fdm_run: bad buffers or step counts");
  if (n_steps % save_every != 0)
    return fail(PRML_ERR_ARG, "prml_fdm_run: n_steps must be a multiple of save_every");
  if (save_every > 1 && (!work_a || !work_b))
    return fail(PRML_ERR_ARG, "prml_fdm_run: strided output needs two work buffers");
  if (base->elem_bytes != 4 && base->elem_bytes != 8)
    return fail(PRML_ERR_ARG, "prml_fdm_run: elem_bytes must be 4 or 8");
  const int gx = (base->ny + tile_y - 1) / tile_y;
  const int gy = (base->nx + tile_x - 1) / tile_x;
  prml_step_params p = *base;
  const size_t ebytes = (size_t)base->elem_bytes;
  const char* cur = static_cast<const char*>(y0);
  long long cur_bstride = y0_bstride;
  int ping = 0;
  for (long long s = 1; s <= n_steps; ++s) {
    char* out;
    long long out_bstride;
    if (s % save_every == 0) {
      out = static_cast<char*>(traj) + (size_t)((s / save_every) - 1) * traj_step_stride * ebytes;
      out_bstride = traj_bstride;
    } else {
      out = static_cast<char*>(ping ? work_b : work_a);
      ping ^= 1;
      out_bstride = work_bstride;
    }
    p.in = cur;
    p.in_bstride = cur_bstride;
    p.out = out;
    p.out_bstride = out_bstride;
    p.t = t0 + (double)(s - 1) * dt;
    p.dt = dt;
    rc = launch_step(k, block, gx, gy, p.batch, &p, static_cast<CUstream>(stream));
    if (rc) return rc;
    cur = out;
    cur_bstride = out_bstride;
  }
  return PRML_OK;
}

int prml_fdm_rhs(void* kernel, int block, int tile_x, int tile_y, const prml_step_params* base,
                 const void* y, long long y_bstride, void* f, long long f_bstride, double t,
                 void* stream) {
  Kernel* k = static_cast<Kernel*>(kernel);
  if (!k) return fail(PRML_ERR_ARG, "prml_fdm_rhs: null kernel");
  int rc = check_geometry(base, tile_x, tile_y, block);
  if (rc) return rc;
  if (!y || !f) return fail(PRML_ERR_ARG, "prml_fdm_rhs: null buffer");
  prml_step_params p = *base;
  p.in = y;
  p.in_bstride = y_bstride;
  p.out = f;
  p.out_bstride = f_bstride;
  p.t = t;
  const int gx = (base->ny + tile_y - 1) / tile_y;
  const int gy = (base->nx + tile_x - 1) / tile_x;
  return launch_step(k, block, gx, gy, p.batch, &p, static_cast<CUstream>(stream));
}

}  // extern "C"
