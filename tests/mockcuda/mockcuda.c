/*
 * mockcuda.c - host-only stand-in for the CUDA runtime calls of libqd.
 *
 * TEST INFRASTRUCTURE.  Preloaded (LD_PRELOAD) into a child process on a machine
 * without a GPU, it lets the library's host engine run: device memory is host
 * memory, copies are memcpy, kernel and graph launches do nothing, events report
 * 10 us.  What it checks is the host logic (validation, session layout and reuse,
 * step scheduling, callbacks, the autotuner's cache), not numerics.
 */
#include <stdlib.h>
#include <string.h>

typedef int cudaError_t;
typedef void *cudaStream_t;
typedef struct {
  unsigned x, y, z;
} mock_dim3;

static int g_launches = 0, g_graph_launches = 0;
int mock_launches(void) { return g_launches; }
int mock_graph_launches(void) { return g_graph_launches; }

cudaError_t cudaGetDeviceCount(int *n) { *n = 1; return 0; }
cudaError_t cudaGetDevice(int *d) { *d = 0; return 0; }
cudaError_t cudaSetDevice(int d) { (void)d; return 0; }
cudaError_t cudaDeviceGetAttribute(int *v, int attr, int dev) {
  (void)attr;
  (void)dev;
  *v = 152;
  return 0;
}
cudaError_t cudaStreamCreateWithFlags(cudaStream_t *s, unsigned f) {
  (void)f;
  *s = malloc(8);
  return 0;
}
cudaError_t cudaStreamDestroy(cudaStream_t s) { free(s); return 0; }
cudaError_t cudaStreamSynchronize(cudaStream_t s) { (void)s; return 0; }
cudaError_t cudaDeviceSynchronize(void) { return 0; }
cudaError_t cudaMalloc(void **p, size_t n) {
  *p = calloc(1, n ? n : 1);
  return *p ? 0 : 2;
}
cudaError_t cudaFree(void *p) { free(p); return 0; }
cudaError_t cudaMemcpyAsync(void *d, const void *s, size_t n, int k, cudaStream_t st) {
  (void)k;
  (void)st;
  memmove(d, s, n);
  return 0;
}
cudaError_t cudaMemcpy(void *d, const void *s, size_t n, int k) {
  (void)k;
  memmove(d, s, n);
  return 0;
}
cudaError_t cudaMemsetAsync(void *d, int v, size_t n, cudaStream_t st) {
  (void)st;
  memset(d, v, n);
  return 0;
}
cudaError_t cudaMemset(void *d, int v, size_t n) { memset(d, v, n); return 0; }
cudaError_t cudaGetLastError(void) { return 0; }
const char *cudaGetErrorString(cudaError_t e) { (void)e; return "mock CUDA runtime"; }
cudaError_t cudaFuncSetAttribute(const void *f, int a, int v) {
  (void)f;
  (void)a;
  (void)v;
  return 0;
}
cudaError_t cudaLaunchKernel(const void *f, mock_dim3 g, mock_dim3 b, void **args, size_t sm, cudaStream_t s) {
  (void)f;
  (void)g;
  (void)b;
  (void)args;
  (void)sm;
  (void)s;
  g_launches++;
  return 0;
}
cudaError_t cudaLaunchKernelExC(const void *cfg, const void *f, void **args) {
  (void)cfg;
  (void)f;
  (void)args;
  g_launches++;
  return 0;
}
cudaError_t cudaEventCreate(void **e) { *e = malloc(8); return 0; }
cudaError_t cudaEventCreateWithFlags(void **e, unsigned flags) { (void)flags; *e = malloc(8); return 0; }
cudaError_t cudaStreamWaitEvent(cudaStream_t s, void *e, unsigned flags) { (void)s; (void)e; (void)flags; return 0; }
cudaError_t cudaMallocHost(void **p, size_t n) { *p = calloc(1, n ? n : 1); return *p ? 0 : 2; }
cudaError_t cudaFreeHost(void *p) { free(p); return 0; }
cudaError_t cudaHostAlloc(void **p, size_t n, unsigned flags) { (void)flags; *p = calloc(1, n ? n : 1); return *p ? 0 : 2; }
cudaError_t cudaEventDestroy(void *e) { free(e); return 0; }
cudaError_t cudaEventRecord(void *e, cudaStream_t s) { (void)e; (void)s; return 0; }
cudaError_t cudaEventSynchronize(void *e) { (void)e; return 0; }
cudaError_t cudaEventElapsedTime(float *ms, void *a, void *b) {
  (void)a;
  (void)b;
  *ms = 0.01f;
  return 0;
}
cudaError_t cudaGetSymbolAddress(void **p, const void *sym) { *p = (void *)sym; return 0; }
cudaError_t cudaStreamBeginCapture(cudaStream_t s, int mode) { (void)s; (void)mode; return 0; }
cudaError_t cudaStreamEndCapture(cudaStream_t s, void **g) { (void)s; *g = malloc(8); return 0; }
cudaError_t cudaGraphInstantiate(void **e, void *g, unsigned long long f) {
  (void)g;
  (void)f;
  *e = malloc(8);
  return 0;
}
cudaError_t cudaGraphDestroy(void *g) { free(g); return 0; }
cudaError_t cudaGraphExecDestroy(void *e) { free(e); return 0; }
cudaError_t cudaGraphLaunch(void *e, cudaStream_t s) { (void)e; (void)s; g_launches++; g_graph_launches++; return 0; }
