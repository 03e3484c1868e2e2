/*
 * A C host that drives FDM steps through the C ABI alone (no Python at run
 * time): the binding a C or C++ caller of the library writes.
 *
 * Input (a directory written by tests/test_gpu_c_host.py from a plan of
 * this package, as a C host would write it once per equation):
 *   run.txt     cubin path, kernel name, shared-memory bytes, threads,
 *               tile rows, tile columns, TMA box rows and columns,
 *               components, steps, dt
 *   params.bin  a prml_step_params whose pointer fields this program fills
 *   dir.bin, neu.bin     Dirichlet / Neumann face tables (state precision)
 *   c0.bin, c1.bin, cz.bin        vertex coordinates (float64)
 *   c0f.bin, c1f.bin, czf.bin     their float32 copies
 *   y0.bin      the initial state, float64 (*vertices, C), C order
 * Output: out.bin, the state after the last step, float64 (*vertices, C).
 *
 * Calls: prml_abi_version, prml_step_params_size, prml_module_load,
 * prml_module_kernel, prml_pack, prml_fdm_run, prml_unpack, prml_last_error.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime.h>

#include "pararealml_gb300.h"

static void* read_all(const char* dir, const char* name, size_t* size) {
  char path[4096];
  snprintf(path, sizeof(path), "%s/%s", dir, name);
  FILE* f = fopen(path, "rb");
  if (!f) {
    fprintf(stderr, "cannot open %s\n", path);
    exit(2);
  }
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  void* buf = malloc(n > 0 ? (size_t)n : 1);
  if (n > 0 && fread(buf, 1, (size_t)n, f) != (size_t)n) {
    fprintf(stderr, "short read of %s\n", path);
    exit(2);
  }
  fclose(f);
  *size = (size_t)n;
  return buf;
}

static void* upload(const char* dir, const char* name) {
  size_t n = 0;
  void* host = read_all(dir, name, &n);
  void* dev = NULL;
  if (cudaMalloc(&dev, n > 0 ? n : 16) != cudaSuccess || cudaMemcpy(dev, host, n, cudaMemcpyHostToDevice) != cudaSuccess) {
    fprintf(stderr, "upload of %s failed\n", name);
    exit(2);
  }
  free(host);
  return dev;
}

static void check(int rc, const char* what) {
  if (rc != PRML_OK) {
    fprintf(stderr, "%s: error %d: %s\n", what, rc, prml_last_error());
    exit(3);
  }
}

int main(int argc, char** argv) {
  if (argc != 2) {
    fprintf(stderr, "usage: %s <run directory>\n", argv[0]);
    return 2;
  }
  const char* dir = argv[1];
  char cubin[4096], kernel_name[256];
  int smem, threads, tile_rows, tile_cols, box_rows, box_cols, comps;
  long long n_steps;
  double dt;
  char path[4096];
  snprintf(path, sizeof(path), "%s/run.txt", dir);
  FILE* f = fopen(path, "r");
  if (!f || fscanf(f, "%4095s %255s %d %d %d %d %d %d %d %lld %lf", cubin, kernel_name, &smem, &threads, &tile_rows,
                   &tile_cols, &box_rows, &box_cols, &comps, &n_steps, &dt) != 11) {
    fprintf(stderr, "bad run.txt\n");
    return 2;
  }
  fclose(f);
  if (prml_abi_version() != PRML_ABI_VERSION) {
    fprintf(stderr, "ABI version mismatch\n");
    return 3;
  }

  size_t n = 0;
  void* blob = read_all(dir, "params.bin", &n);
  if (n != sizeof(prml_step_params) || prml_step_params_size() != (int)sizeof(prml_step_params)) {
    fprintf(stderr, "prml_step_params is %zu bytes here, %zu in the file\n", sizeof(prml_step_params), n);
    return 3;
  }
  prml_step_params p;
  memcpy(&p, blob, sizeof(p));
  free(blob);
  p.dirichlet = upload(dir, "dir.bin");
  p.neumann = upload(dir, "neu.bin");
  p.coord0 = (const double*)upload(dir, "c0.bin");
  p.coord1 = (const double*)upload(dir, "c1.bin");
  p.coord2 = (const double*)upload(dir, "cz.bin");
  p.coord0_f = (const float*)upload(dir, "c0f.bin");
  p.coord1_f = (const float*)upload(dir, "c1f.bin");
  p.coord2_f = (const float*)upload(dir, "czf.bin");
  p.t_offset = NULL;
  p.bc_inst_slot = NULL;
  int* status = NULL;
  cudaMalloc((void**)&status, sizeof(int));
  cudaMemset(status, 0, sizeof(int));
  p.status = status;

  const long long inst = (long long)comps * p.nx * p.pitch; /* one instance, one plane per component */
  const long long nv = (long long)p.nx * p.ny;
  void* y0 = upload(dir, "y0.bin");
  void *state0 = NULL, *traj = NULL, *work = NULL;
  double* out = NULL;
  cudaMalloc(&state0, (size_t)(inst * p.elem_bytes));
  cudaMalloc(&traj, (size_t)(n_steps * inst * p.elem_bytes));
  cudaMalloc(&work, (size_t)(2 * inst * p.elem_bytes));
  cudaMalloc((void**)&out, (size_t)(nv * comps * 8));
  cudaMemset(state0, 0, (size_t)(inst * p.elem_bytes)); /* the row padding */

  void* module = NULL;
  void* kernel = NULL;
  check(prml_module_load(cubin, &module), "prml_module_load");
  check(prml_module_kernel(module, kernel_name, smem, &kernel), "prml_module_kernel");
  cudaStream_t stream;
  cudaStreamCreate(&stream);
  check(prml_pack((const double*)y0, state0, p.elem_bytes, 1, comps, p.nx, p.ny, p.pitch, nv * comps, inst, 0, stream),
        "prml_pack");
  check(prml_fdm_run(kernel, threads, tile_rows, tile_cols, box_rows, box_cols, comps, &p, state0, inst, traj, inst,
                     inst, work, (char*)work + inst * p.elem_bytes, inst, n_steps, 1, 0.0, dt, stream),
        "prml_fdm_run");
  check(prml_unpack((const char*)traj + (n_steps - 1) * inst * p.elem_bytes, p.elem_bytes, out, 1, comps, p.nx, p.ny,
                    p.pitch, inst, nv * comps, 0, stream),
        "prml_unpack");
  if (cudaStreamSynchronize(stream) != cudaSuccess) {
    fprintf(stderr, "stream: %s\n", cudaGetErrorString(cudaGetLastError()));
    return 3;
  }
  int flag = 0;
  cudaMemcpy(&flag, status, sizeof(int), cudaMemcpyDeviceToHost);
  if (flag) {
    fprintf(stderr, "a kernel timed out in a bounded wait\n");
    return 3;
  }
  double* host = (double*)malloc((size_t)(nv * comps * 8));
  cudaMemcpy(host, out, (size_t)(nv * comps * 8), cudaMemcpyDeviceToHost);
  snprintf(path, sizeof(path), "%s/out.bin", dir);
  f = fopen(path, "wb");
  fwrite(host, 8, (size_t)(nv * comps), f);
  fclose(f);
  free(host);
  check(prml_kernel_free(kernel), "prml_kernel_free");
  check(prml_module_unload(module), "prml_module_unload");
  printf("ok %lld steps\n", n_steps);
  return 0;
}
