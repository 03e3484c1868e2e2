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
  CUresult (*LaunchKernelEx)(const CUlaunchConfig*, CUfunction, void**, void**) = nullptr; /* optional */
  CUresult (*TensorMapEncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill) = nullptr;
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
         bind(h, "cuLaunchKernel", d.LaunchKernel) &&
         bind(h, "cuTensorMapEncodeTiled", d.TensorMapEncodeTiled);
  bind(h, "cuLaunchKernelEx", d.LaunchKernelEx);
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
  int grid_cap = 0; /* CTAs resident on the whole GPU at once (persistent grid) */
};

}  // namespace

int prml_set_error(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

void* prml_current_context() {
  if (!driver()) return nullptr;
  CUcontext ctx = nullptr;
  if (g_drv.CtxGetCurrent(&ctx) != CUDA_SUCCESS) return nullptr;
  return ctx;
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
  /* the step kernels stage everything in shared memory and gain nothing
   * from L1: ask for the largest shared-memory carveout (a preference) */
  g_drv.FuncSetAttribute(k->fn, CU_FUNC_ATTRIBUTE_PREFERRED_SHARED_MEMORY_CARVEOUT, 100);
  /* opt in to the requested dynamic size whatever it is: a kernel with
   * static shared memory too (the multi-round kernels' group tables) can
   * exceed the 48 KB default with less than 48 KB of dynamic memory */
  if (smem_bytes > 0) {
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

/* 5D tensor map over [slot][instance][C][row][col] of a state buffer. */
static int encode_state_map(CUtensorMap* map, const prml_step_params* p, const void* base,
                            long long bstride, long long slot_stride, int slots, int box_rows,
                            int box_cols, int comps) {
  if (!driver()) return fail(PRML_ERR_CUDA, "cannot load the CUDA driver (libcuda.so.1)");
  const cuuint64_t e = (cuuint64_t)p->elem_bytes;
  cuuint64_t dims[5] = {(cuuint64_t)p->ny, (cuuint64_t)p->nx, (cuuint64_t)comps,
                        (cuuint64_t)p->batch, (cuuint64_t)slots};
  cuuint64_t strides[4] = {(cuuint64_t)p->pitch * e, (cuuint64_t)p->cstride * e,
                           (cuuint64_t)bstride * e, (cuuint64_t)slot_stride * e};
  cuuint32_t box[5] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows, (cuuint32_t)comps, 1, 1};
  if (p->nz > 1) {
    /* 3D: (columns, rows, planes, components, instance x slot); the
     * instance and slot dimensions merge, which needs slots laid out
     * batch instances apart */
    if (slots > 1 && slot_stride != bstride * p->batch)
      return fail(PRML_ERR_ARG, "3D states need slots batch instances apart");
    const int bp = p->box_planes;
    if (bp < 1 || bp > 256) return fail(PRML_ERR_ARG, "bad TMA box depth");
    dims[0] = (cuuint64_t)p->ny;
    dims[1] = (cuuint64_t)p->nx;
    dims[2] = (cuuint64_t)p->nz;
    dims[3] = (cuuint64_t)comps;
    dims[4] = (cuuint64_t)p->batch * (cuuint64_t)slots;
    strides[0] = (cuuint64_t)p->pitch * e;
    strides[1] = (cuuint64_t)p->nx * (cuuint64_t)p->pitch * e;
    strides[2] = (cuuint64_t)p->cstride * e;
    strides[3] = (cuuint64_t)bstride * e;
    box[0] = (cuuint32_t)box_cols;
    box[1] = (cuuint32_t)box_rows;
    box[2] = (cuuint32_t)bp;
    box[3] = (cuuint32_t)comps;
    box[4] = 1;
  }
  cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  for (int i = 0; i < 4; ++i)
    if (strides[i] % 16 != 0) return fail(PRML_ERR_ARG, "state strides must be multiples of 16 bytes");
  if ((reinterpret_cast<unsigned long long>(base) & 15ull) != 0)
    return fail(PRML_ERR_ARG, "state buffers must be 16-byte aligned");
  if (box_cols < 1 || box_cols > 256 || box_rows < 1 || box_rows > 256 || comps > 256 ||
      ((long long)box_cols * p->elem_bytes) % 16 != 0)
    return fail(PRML_ERR_ARG, "bad TMA box");
  CUresult r = g_drv.TensorMapEncodeTiled(
      map, p->elem_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 5,
      const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
      CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(PRML_ERR_CUDA, std::string("cuTensorMapEncodeTiled: ") + cu_name(r));
  return PRML_OK;
}

int prml_tensor_map_tiled(CUtensorMap* map, CUtensorMapDataType dtype, unsigned rank, const void* base,
                          const unsigned long long* dims, const unsigned long long* strides,
                          const unsigned* box, int swizzle_bytes) {
  CUtensorMapSwizzle swz;
  switch (swizzle_bytes) {
    case 0: swz = CU_TENSOR_MAP_SWIZZLE_NONE; break;
    case 32: swz = CU_TENSOR_MAP_SWIZZLE_32B; break;
    case 64: swz = CU_TENSOR_MAP_SWIZZLE_64B; break;
    case 128: swz = CU_TENSOR_MAP_SWIZZLE_128B; break;
    default: return fail(PRML_ERR_ARG, "swizzle must be 0, 32, 64 or 128 bytes");
  }
  if (!driver()) return fail(PRML_ERR_CUDA, "cannot load the CUDA driver (libcuda.so.1)");
  if (rank < 1 || rank > 5) return fail(PRML_ERR_ARG, "tensor map rank must be 1..5");
  cuuint64_t d[5], st[4];
  cuuint32_t bx[5], es[5];
  for (unsigned i = 0; i < rank; ++i) {
    d[i] = (cuuint64_t)dims[i];
    bx[i] = (cuuint32_t)box[i];
    es[i] = 1;
  }
  for (unsigned i = 0; i + 1 < rank; ++i) {
    st[i] = (cuuint64_t)strides[i];
    if (st[i] % 16 != 0) return fail(PRML_ERR_ARG, "tensor map strides must be multiples of 16 bytes");
  }
  if ((reinterpret_cast<unsigned long long>(base) & 15ull) != 0)
    return fail(PRML_ERR_ARG, "tensor map base must be 16-byte aligned");
  CUresult r = g_drv.TensorMapEncodeTiled(map, dtype, rank, const_cast<void*>(base), d, st, bx, es,
                                          CU_TENSOR_MAP_INTERLEAVE_NONE, swz,
                                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(PRML_ERR_CUDA, std::string("cuTensorMapEncodeTiled: ") + cu_name(r));
  return PRML_OK;
}

/* Grid of the persistent step kernels: every CTA that can be resident at
 * once (SMs x blocks per SM), but no more than there are tiles. */
static int persistent_grid(Kernel* k, int block, const prml_step_params* base, int tile_x,
                           int tile_y, int* grid) {
  if (k->grid_cap == 0) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return fail(PRML_ERR_CUDA, std::string("device query: ") + cudaGetErrorString(e));
    CUresult r = g_drv.OccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k->fn, block, k->smem);
    if (r != CUDA_SUCCESS) return fail(PRML_ERR_CUDA, std::string("occupancy: ") + cu_name(r));
    if (per_sm < 1) return fail(PRML_ERR_ARG, "step kernel does not fit on an SM");
    k->grid_cap = sms * per_sm;
  }
  const int tz = base->tile_z > 0 ? base->tile_z : 1;
  const int nz = base->nz > 0 ? base->nz : 1;
  const long long tiles = (long long)((base->ny + tile_y - 1) / tile_y) *
                          ((base->nx + tile_x - 1) / tile_x) * ((nz + tz - 1) / tz) * base->batch;
  long long cap = k->grid_cap;
  if (base->max_ctas > 0 && base->max_ctas < cap) cap = base->max_ctas;
  if (tiles + cap >= (1LL << 31)) return fail(PRML_ERR_ARG, "too many tiles for one launch (2^31)");
  /* as many rounds of tiles as the resident CTAs need, and the tiles spread
   * evenly over them: no CTA walks more tiles than another plus one */
  const long long rounds = (tiles + cap - 1) / cap;
  const long long g = (tiles + rounds - 1) / rounds;
  *grid = (int)(g < 1 ? 1 : g);
  return PRML_OK;
}

/* Step launches overlap their predecessor (programmatic dependent launch):
 * a step kernel lets the next launch start as soon as all of its CTAs run,
 * and every step kernel waits (griddepcontrol.wait) for its predecessor to
 * complete before it touches global memory, so only CTA dispatch and setup
 * overlap.  On by default; prml_set_step_overlap switches it. */
static int g_step_overlap = 1;

int prml_set_step_overlap(int enabled) {
  const int prev = g_step_overlap;
  g_step_overlap = enabled ? 1 : 0;
  return prev;
}

static int launch_step(Kernel* k, int block, int grid, prml_step_params* p, CUtensorMap* map,
                       CUstream stream) {
  void* args[] = {p, map};
  CUresult r;
  if (g_step_overlap && g_drv.LaunchKernelEx) {
    CUlaunchAttribute attr[1];
    std::memset(attr, 0, sizeof(attr));
    attr[0].id = CU_LAUNCH_ATTRIBUTE_PROGRAMMATIC_STREAM_SERIALIZATION;
    attr[0].value.programmaticStreamSerializationAllowed = 1;
    CUlaunchConfig cfg;
    std::memset(&cfg, 0, sizeof(cfg));
    cfg.gridDimX = (unsigned)grid;
    cfg.gridDimY = cfg.gridDimZ = 1;
    cfg.blockDimX = (unsigned)block;
    cfg.blockDimY = cfg.blockDimZ = 1;
    cfg.sharedMemBytes = (unsigned)k->smem;
    cfg.hStream = stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    r = g_drv.LaunchKernelEx(&cfg, k->fn, args, nullptr);
    if (r != CUDA_SUCCESS) return fail(PRML_ERR_CUDA, std::string("cuLaunchKernelEx: ") + cu_name(r));
    return PRML_OK;
  }
  r = g_drv.LaunchKernel(k->fn, grid, 1, 1, block, 1, 1, k->smem, stream, args, nullptr);
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
  if (base->elem_bytes != 4 && base->elem_bytes != 8)
    return fail(PRML_ERR_ARG, "elem_bytes must be 4 or 8");
  long long gy = (base->nx + tile_x - 1) / tile_x;
  if (gy > 65535) return fail(PRML_ERR_ARG, "too many row tiles");
  return PRML_OK;
}

int prml_fdm_run(void* kernel, int block, int tile_x, int tile_y, int box_rows, int box_cols,
                 int comps, const prml_step_params* base, const void* y0, long long y0_bstride,
                 void* traj, long long traj_bstride, long long traj_step_stride,
                 void* work_a, void* work_b, long long work_bstride, long long n_steps,
                 int save_every, double t0, double dt, void* stream) {
  Kernel* k = static_cast<Kernel*>(kernel);
  if (!k) return fail(PRML_ERR_ARG, "prml_fdm_run: null kernel");
  int rc = check_geometry(base, tile_x, tile_y, block);
  if (rc) return rc;
  if (!y0 || !traj || n_steps < 0 || save_every < 1 || comps < 1)
    return fail(PRML_ERR_ARG, "prml_fdm_run: bad buffers or step counts");
  if (n_steps % save_every != 0)
    return fail(PRML_ERR_ARG, "prml_fdm_run: n_steps must be a multiple of save_every");
  if (save_every > 1 && (!work_a || !work_b))
    return fail(PRML_ERR_ARG, "prml_fdm_run: strided output needs two work buffers");
  if (n_steps == 0) return PRML_OK;
  int grid = 0;
  rc = persistent_grid(k, block, base, tile_x, tile_y, &grid);
  if (rc) return rc;
  const long long n_save = n_steps / save_every;
  prml_step_params p = *base;
  const size_t ebytes = (size_t)base->elem_bytes;

  CUtensorMap map_y0, map_traj, map_wa, map_wb;
  rc = encode_state_map(&map_y0, base, y0, y0_bstride, y0_bstride * base->batch, 1, box_rows,
                        box_cols, comps);
  if (rc) return rc;
  rc = encode_state_map(&map_traj, base, traj, traj_bstride, traj_step_stride, (int)n_save,
                        box_rows, box_cols, comps);
  if (rc) return rc;
  if (save_every > 1) {
    rc = encode_state_map(&map_wa, base, work_a, work_bstride, work_bstride * base->batch, 1,
                          box_rows, box_cols, comps);
    if (rc) return rc;
    rc = encode_state_map(&map_wb, base, work_b, work_bstride, work_bstride * base->batch, 1,
                          box_rows, box_cols, comps);
    if (rc) return rc;
  }

  /* A temporally blocked kernel (tb_max > 1) takes up to tb_max steps per
   * launch; its intermediate steps go straight to their trajectory slots
   * (or nowhere when they are not saved) and only the last step of a launch
   * is stored through `out`, so the step-to-buffer assignment below is the
   * same as for one step per launch. */
  const int tb = base->tb_max > 1 ? base->tb_max : 1;
  if (tb > PRML_TB_MAX) return fail(PRML_ERR_ARG, "prml_fdm_run: tb_max above PRML_TB_MAX");
  p.tb_bstride = traj_bstride;
  const char* cur = static_cast<const char*>(y0);
  long long cur_bstride = y0_bstride; /* instance stride of `cur` */
  CUtensorMap* cur_map = &map_y0;
  int cur_slot = 0;
  int ping = 0;
  for (long long s0 = 1; s0 <= n_steps; s0 += tb) {
    const long long s_last = (s0 + tb - 1 <= n_steps) ? s0 + tb - 1 : n_steps;
    p.tb_steps = (int)(s_last - s0 + 1);
    for (int j = 0; j < PRML_TB_MAX - 1; ++j) p.tb_out[j] = nullptr;
    for (long long s = s0; s < s_last; ++s)
      if (s % save_every == 0)
        p.tb_out[s - s0] = static_cast<char*>(traj) + (size_t)(s / save_every - 1) * traj_step_stride * ebytes;
    char* out;
    long long out_bstride;
    CUtensorMap* out_map;
    int out_slot;
    if (s_last % save_every == 0) {
      out_slot = (int)(s_last / save_every - 1);
      out = static_cast<char*>(traj) + (size_t)out_slot * traj_step_stride * ebytes;
      out_bstride = traj_bstride;
      out_map = &map_traj;
    } else {
      out = static_cast<char*>(ping ? work_b : work_a);
      out_map = ping ? &map_wb : &map_wa;
      out_slot = 0;
      ping ^= 1;
      out_bstride = work_bstride;
    }
    p.in = cur;
    p.in_bstride = cur_bstride;
    p.in_slot = cur_slot;
    p.out = out;
    p.out_bstride = out_bstride;
    p.t = t0 + (double)(s0 - 1) * dt;
    p.dt = dt;
    p.dt_f = (float)dt;
    p.bc_slot0 = base->bc_slot0 + (int)(2 * (s0 - 1));
    rc = launch_step(k, block, grid, &p, cur_map, static_cast<CUstream>(stream));
    if (rc) return rc;
    cur = out;
    cur_bstride = out_bstride;
    cur_map = out_map;
    cur_slot = out_slot;
  }
  return PRML_OK;
}

/* ---- multi-round launches --------------------------------------------- */

static long long multi_maps_offset(int n_groups) {
  return ((long long)n_groups * (long long)sizeof(prml_multi_group) + 127) / 128 * 128;
}

int prml_multi_group_size(void) { return (int)sizeof(prml_multi_group); }

long long prml_multi_desc_bytes(int n_groups) {
  if (n_groups < 1 || n_groups > PRML_MULTI_MAX_GROUPS) return -1;
  return multi_maps_offset(n_groups) + 2LL * n_groups * (long long)sizeof(CUtensorMap);
}

int prml_multi_prepare(const prml_multi_group* groups, int n_groups, int tile_x, int tile_y, int box_rows,
                       int box_cols, int comps, void* desc, long long desc_bytes) {
  if (!groups || !desc || n_groups < 1 || n_groups > PRML_MULTI_MAX_GROUPS)
    return fail(PRML_ERR_ARG, "prml_multi_prepare: bad groups or descriptor buffer");
  if (desc_bytes < prml_multi_desc_bytes(n_groups))
    return fail(PRML_ERR_ARG, "prml_multi_prepare: descriptor buffer too small");
  if ((reinterpret_cast<unsigned long long>(desc) & 127ull) != 0)
    return fail(PRML_ERR_ARG, "prml_multi_prepare: descriptor buffer must be 128-byte aligned");
  std::vector<prml_multi_group> g(groups, groups + n_groups);
  std::vector<CUtensorMap> maps(2 * (size_t)n_groups);
  for (int i = 0; i < n_groups; ++i) {
    prml_multi_group& gr = g[i];
    int rc = check_geometry(&gr.p, tile_x, tile_y, 32);
    if (rc) return rc;
    if (gr.p.nz > 1) return fail(PRML_ERR_UNSUPPORTED, "prml_multi_prepare: 3D meshes take one launch per step");
    if (!gr.first || !gr.main || gr.n_steps < 1 || gr.slot_stride < 1)
      return fail(PRML_ERR_ARG, "prml_multi_prepare: bad group buffers or step count");
    if (gr.p.in_bstride != gr.p.out_bstride || gr.p.in_bstride < 1)
      return fail(PRML_ERR_ARG, "prml_multi_prepare: first and main must share the instance stride");
    if (gr.ping_pong && gr.slot_stride < gr.p.in_bstride * gr.p.batch)
      return fail(PRML_ERR_ARG, "prml_multi_prepare: slots overlap");
    gr.tiles_x = (gr.p.ny + tile_y - 1) / tile_y;
    gr.tiles_y = (gr.p.nx + tile_x - 1) / tile_x;
    if ((long long)gr.tiles_x * gr.tiles_y * gr.p.batch >= (1LL << 30))
      return fail(PRML_ERR_ARG, "prml_multi_prepare: too many tiles");
    gr.p.max_ctas = 0;
    gr.p.bc_inst_slot = nullptr;
    gr.p.tb_max = 1;
    gr.p.tb_steps = 1;
    const int slots = gr.ping_pong ? 2 : gr.n_steps;
    rc = encode_state_map(&maps[2 * i], &gr.p, gr.first, gr.p.in_bstride, gr.p.in_bstride * gr.p.batch, 1,
                          box_rows, box_cols, comps);
    if (rc) return rc;
    rc = encode_state_map(&maps[2 * i + 1], &gr.p, gr.main, gr.p.in_bstride, gr.slot_stride, slots, box_rows,
                          box_cols, comps);
    if (rc) return rc;
  }
  char* d = static_cast<char*>(desc);
  cudaError_t e = cudaMemcpy(d, g.data(), g.size() * sizeof(prml_multi_group), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(d + multi_maps_offset(n_groups), maps.data(), maps.size() * sizeof(CUtensorMap),
                   cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return fail(PRML_ERR_CUDA, std::string("prml_multi_prepare: ") + cudaGetErrorString(e));
  return PRML_OK;
}

int prml_multi_launch(void* kernel, int block, const void* desc, int n_groups, int n_rounds,
                      long long max_round_tiles, unsigned long long* barrier, int* status, int max_ctas,
                      void* stream) {
  Kernel* k = static_cast<Kernel*>(kernel);
  if (!k || !desc || !barrier || n_groups < 1 || n_groups > PRML_MULTI_MAX_GROUPS || n_rounds < 0 ||
      max_round_tiles < 1 || block < 32 || block > 1024)
    return fail(PRML_ERR_ARG, "prml_multi_launch: bad argument");
  if (n_rounds == 0) return PRML_OK;
  if (!driver()) return fail(PRML_ERR_CUDA, "cannot load the CUDA driver (libcuda.so.1)");
  if (!g_drv.LaunchKernelEx) return fail(PRML_ERR_UNSUPPORTED, "prml_multi_launch: cuLaunchKernelEx missing");
  if (k->grid_cap == 0) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return fail(PRML_ERR_CUDA, std::string("device query: ") + cudaGetErrorString(e));
    PRML_CU(g_drv.OccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k->fn, block, k->smem));
    if (per_sm < 1) return fail(PRML_ERR_ARG, "multi-round kernel does not fit on an SM");
    k->grid_cap = sms * per_sm;
  }
  /* every CTA must be resident at once (the rounds meet at a grid barrier):
   * at most one CTA per resident slot, and no more CTAs than the largest
   * round has tiles */
  long long grid = k->grid_cap;
  if (max_ctas > 0 && max_ctas < grid) grid = max_ctas;
  if (max_round_tiles < grid) grid = max_round_tiles;
  prml_multi_params mp;
  std::memset(&mp, 0, sizeof(mp));
  mp.groups = static_cast<const prml_multi_group*>(desc);
  mp.maps = static_cast<const char*>(desc) + multi_maps_offset(n_groups);
  mp.barrier = barrier;
  mp.status = status;
  mp.n_groups = n_groups;
  mp.n_rounds = n_rounds;
  CUstream st = static_cast<CUstream>(stream);
  cudaError_t e = cudaMemsetAsync(barrier, 0, sizeof(unsigned long long), static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return fail(PRML_ERR_CUDA, std::string("prml_multi_launch: ") + cudaGetErrorString(e));
  void* args[] = {&mp};
  CUlaunchAttribute attr[1];
  std::memset(attr, 0, sizeof(attr));
  attr[0].id = CU_LAUNCH_ATTRIBUTE_COOPERATIVE;
  attr[0].value.cooperative = 1;
  CUlaunchConfig cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.gridDimX = (unsigned)grid;
  cfg.gridDimY = cfg.gridDimZ = 1;
  cfg.blockDimX = (unsigned)block;
  cfg.blockDimY = cfg.blockDimZ = 1;
  cfg.sharedMemBytes = (unsigned)k->smem;
  cfg.hStream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  CUresult r = g_drv.LaunchKernelEx(&cfg, k->fn, args, nullptr);
  if (r != CUDA_SUCCESS) return fail(PRML_ERR_CUDA, std::string("cuLaunchKernelEx (cooperative): ") + cu_name(r));
  return PRML_OK;
}

int prml_fdm_rhs(void* kernel, int block, int tile_x, int tile_y, int box_rows, int box_cols,
                 int comps, const prml_step_params* base, const void* y, long long y_bstride,
                 void* f, long long f_bstride, double t, void* stream) {
  Kernel* k = static_cast<Kernel*>(kernel);
  if (!k) return fail(PRML_ERR_ARG, "prml_fdm_rhs: null kernel");
  int rc = check_geometry(base, tile_x, tile_y, block);
  if (rc) return rc;
  if (!y || !f || comps < 1) return fail(PRML_ERR_ARG, "prml_fdm_rhs: null buffer");
  CUtensorMap map;
  rc = encode_state_map(&map, base, y, y_bstride, y_bstride * base->batch, 1, box_rows, box_cols,
                        comps);
  if (rc) return rc;
  prml_step_params p = *base;
  p.in = y;
  p.in_slot = 0;
  p.out = f;
  p.out_bstride = f_bstride;
  p.t = t;
  int grid = 0;
  rc = persistent_grid(k, block, base, tile_x, tile_y, &grid);
  if (rc) return rc;
  return launch_step(k, block, grid, &p, &map, static_cast<CUstream>(stream));
}

}  // extern "C"
