/*
 * arch_gb300.c -- single-rank GPU arch layer of the flow host driver
 * (include/flow_arch.h): params parsing, device allocation, uniform mesh
 * set-up, problem set-up (the params boxes, rasterised on the device by the
 * kernel set's gb300_fill_boxes) and the VisIt dump.  Compiled into
 * libflow_gb300_arch.so, which links libflow_gb300.so.
 */
#include <cuda_runtime.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/flow_arch.h"
#include "../../include/flow_gb300.h"

struct Profile compute_profile;
struct Profile comms_profile;

static void cuda_or_die(cudaError_t err, const char* what) {
  if (err != cudaSuccess) {
    TERMINATE("%s failed: %s\n", what, cudaGetErrorString(err));
  }
}

/* ---- params ------------------------------------------------------------- */

/* Finds the line whose first token is `key`; returns the text after it in a
 * static buffer, or NULL. */
static const char* param_line(const char* key, const char* filename) {
  static char line[MAX_STR_LEN];
  FILE* fp = fopen(filename, "r");
  if (!fp) TERMINATE("could not open parameter file %s\n", filename);
  const size_t klen = strlen(key);
  const char* found = NULL;
  while (fgets(line, sizeof(line), fp)) {
    char* p = line;
    while (*p == ' ' || *p == '\t') ++p;
    if (strncmp(p, key, klen) == 0 &&
        (p[klen] == ' ' || p[klen] == '\t' || p[klen] == '\n' ||
         p[klen] == '\r' || p[klen] == '\0')) {
      found = p + klen;
      break;
    }
  }
  fclose(fp);
  return found;
}

int get_int_parameter(const char* key, const char* filename) {
  const char* rest = param_line(key, filename);
  if (!rest) TERMINATE("parameter %s not found in %s\n", key, filename);
  return (int)strtol(rest, NULL, 10);
}

double get_double_parameter(const char* key, const char* filename) {
  const char* rest = param_line(key, filename);
  if (!rest) TERMINATE("parameter %s not found in %s\n", key, filename);
  return strtod(rest, NULL);
}

int get_key_value_parameter(const char* specifier, const char* filename,
                            char* keys, double* values, int* nkeys) {
  *nkeys = 0;
  const char* rest = param_line(specifier, filename);
  if (!rest) return 0;
  char buf[MAX_STR_LEN];
  strncpy(buf, rest, sizeof(buf) - 1);
  buf[sizeof(buf) - 1] = '\0';
  char* save = NULL;
  for (char* tok = strtok_r(buf, " \t\r\n", &save); tok;
       tok = strtok_r(NULL, " \t\r\n", &save)) {
    char* eq = strchr(tok, '=');
    if (!eq || *nkeys >= MAX_KEYS) continue;
    *eq = '\0';
    char* k = &keys[(*nkeys) * (MAX_STR_LEN + 1)];
    strncpy(k, tok, MAX_STR_LEN);
    k[MAX_STR_LEN] = '\0';
    values[*nkeys] = strtod(eq + 1, NULL);
    (*nkeys)++;
  }
  return 1;
}

int strmatch(const char* a, const char* b) { return strcmp(a, b) == 0; }

/* ---- comms (one rank) ----------------------------------------------------- */

void initialise_mpi(int argc, char** argv, int* rank, int* nranks) {
  (void)argc;
  (void)argv;
  *rank = MASTER;
  *nranks = 1;
}

void initialise_comms(Mesh* mesh) {
  for (int k = 0; k < 4; ++k) mesh->neighbours[k] = FLOW_EDGE;
  mesh->x_off = 0;
  mesh->y_off = 0;
}

void initialise_devices(int rank) {
  int count = 0;
  cuda_or_die(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
  if (count == 0) TERMINATE("no CUDA device: the GB300 kernel set has no CPU path\n");
  cuda_or_die(cudaSetDevice(rank % count), "cudaSetDevice");
}

double reduce_all_min(double value) { return value; }
double reduce_all_sum(double value) { return value; }
double reduce_to_master(double value) { return value; }
void barrier(void) { cuda_or_die(cudaDeviceSynchronize(), "cudaDeviceSynchronize"); }

/* ---- memory --------------------------------------------------------------- */

size_t allocate_data(double** buf, size_t len) {
  const size_t bytes = (len ? len : 1) * sizeof(double);
  cuda_or_die(cudaMalloc((void**)buf, bytes), "cudaMalloc");
  cuda_or_die(cudaMemset(*buf, 0, bytes), "cudaMemset");
  return bytes;
}

void deallocate_data(double* buf) { cudaFree(buf); }

size_t allocate_host_data(double** buf, size_t len) {
  *buf = (double*)calloc(len ? len : 1, sizeof(double));
  if (!*buf) TERMINATE("host allocation of %zu doubles failed\n", len);
  return len * sizeof(double);
}

void deallocate_host_data(double* buf) { free(buf); }

void copy_buffer(size_t len, double** src, double** dst, int send) {
  cuda_or_die(cudaMemcpy(*dst, *src, len * sizeof(double),
                         send == SEND ? cudaMemcpyHostToDevice
                                      : cudaMemcpyDeviceToHost),
              "copy_buffer");
}

/* ---- mesh ----------------------------------------------------------------- */

static double* upload(const double* h, size_t n) {
  double* d = NULL;
  cuda_or_die(cudaMalloc((void**)&d, n * sizeof(double)), "cudaMalloc");
  cuda_or_die(cudaMemcpy(d, h, n * sizeof(double), cudaMemcpyHostToDevice),
              "cudaMemcpy");
  return d;
}

void initialise_mesh_2d(Mesh* mesh) {
  const int nx = mesh->local_nx, ny = mesh->local_ny;
  double* ex = (double*)malloc(sizeof(double) * (nx + 1));
  double* ey = (double*)malloc(sizeof(double) * (ny + 1));
  double* dxs = (double*)malloc(sizeof(double) * (nx + 1));
  double* dys = (double*)malloc(sizeof(double) * (ny + 1));
  const double dx = mesh->width / (double)mesh->global_nx;
  const double dy = mesh->height / (double)mesh->global_ny;
  for (int jj = 0; jj <= nx; ++jj) {
    ex[jj] = mesh->width * (double)(mesh->x_off + jj - mesh->pad) / mesh->global_nx;
    dxs[jj] = dx;
  }
  for (int ii = 0; ii <= ny; ++ii) {
    ey[ii] = mesh->height * (double)(mesh->y_off + ii - mesh->pad) / mesh->global_ny;
    dys[ii] = dy;
  }
  mesh->edgex = upload(ex, nx + 1);
  mesh->edgey = upload(ey, ny + 1);
  mesh->edgedx = upload(dxs, nx + 1);
  mesh->celldx = upload(dxs, nx + 1);
  mesh->edgedy = upload(dys, ny + 1);
  mesh->celldy = upload(dys, ny + 1);
  free(ex);
  free(ey);
  free(dxs);
  free(dys);
}

void finalise_mesh(Mesh* mesh) {
  cudaFree(mesh->edgex);
  cudaFree(mesh->edgey);
  cudaFree(mesh->edgedx);
  cudaFree(mesh->edgedy);
  cudaFree(mesh->celldx);
  cudaFree(mesh->celldy);
}

/* The problem boxes of the params file (problem_0, problem_1, ...: density,
 * energy, xpos, ypos, width, height) as rows of 6 doubles; returns the count. */
static int parse_boxes(const char* params, double* boxes, int max_boxes) {
  char* keys = (char*)malloc(MAX_KEYS * (MAX_STR_LEN + 1));
  double values[MAX_KEYS];
  int nb = 0;
  for (int pp = 0;; ++pp) {
    char spec[64];
    snprintf(spec, sizeof(spec), "problem_%d", pp);
    int n = 0;
    if (!get_key_value_parameter(spec, params, keys, values, &n)) break;
    if (nb == max_boxes) TERMINATE("more than %d problem boxes\n", max_boxes);
    double* b = boxes + 6 * nb;
    int have = 0;
    for (int k = 0; k < n; ++k) {
      const char* key = &keys[k * (MAX_STR_LEN + 1)];
      if (strmatch(key, "density")) { b[0] = values[k]; have |= 1; }
      else if (strmatch(key, "energy")) { b[1] = values[k]; have |= 2; }
      else if (strmatch(key, "xpos")) { b[2] = values[k]; have |= 4; }
      else if (strmatch(key, "ypos")) { b[3] = values[k]; have |= 8; }
      else if (strmatch(key, "width")) { b[4] = values[k]; have |= 16; }
      else if (strmatch(key, "height")) { b[5] = values[k]; have |= 32; }
    }
    if (have != 63) TERMINATE("%s needs density energy xpos ypos width height\n", spec);
    ++nb;
  }
  free(keys);
  return nb;
}

void initialise_shared_data_2d(const int local_nx, const int local_ny,
                               const int pad, const double width,
                               const double height, const char* params_filename,
                               const double* edgex, const double* edgey,
                               SharedData* sd) {
  (void)pad;
  (void)width;
  (void)height;
  const size_t nc = (size_t)local_nx * local_ny;
  const size_t nf = (size_t)(local_nx + 1) * (local_ny + 1);
  allocate_data(&sd->pressure, nc);
  allocate_data(&sd->density, nc);
  allocate_data(&sd->density_old, nc);
  allocate_data(&sd->energy, nc);
  allocate_data(&sd->u, nf);
  allocate_data(&sd->v, nf);
  allocate_data(&sd->Qxx, nc);
  allocate_data(&sd->Qyy, nc);
  allocate_data(&sd->reduce_array0, nc);
  allocate_data(&sd->reduce_array1, nc);
  if (!edgex || !edgey) TERMINATE("initialise_mesh_2d must run first\n");
  /* The boxes are rasterised on the device (gb300_fill_boxes): no host
   * arrays and no copies of the fields. */
  double boxes[6 * GB300_MAX_BOXES];
  const int nb = parse_boxes(params_filename, boxes, GB300_MAX_BOXES);
  if (gb300_fill_boxes(local_nx, local_ny, edgex, edgey, boxes, nb, sd->density,
                       sd->energy) != GB300_OK) {
    TERMINATE("problem set-up: %s\n", gb300_last_error_message());
  }
  cuda_or_die(cudaDeviceSynchronize(), "problem set-up");
}

void finalise_shared_data(SharedData* sd) {
  deallocate_data(sd->pressure);
  deallocate_data(sd->density);
  deallocate_data(sd->density_old);
  deallocate_data(sd->energy);
  deallocate_data(sd->u);
  deallocate_data(sd->v);
  deallocate_data(sd->Qxx);
  deallocate_data(sd->Qyy);
  deallocate_data(sd->reduce_array0);
  deallocate_data(sd->reduce_array1);
}

int within_tolerance(const double expected, const double actual,
                     const double tolerance) {
  const double scale = expected != 0.0 ? (expected > 0 ? expected : -expected) : 1.0;
  const double d = actual - expected;
  return (d < 0 ? -d : d) <= tolerance * scale;
}

/* ---- VisIt dump ----------------------------------------------------------
 *
 * write_all_ranks_to_visit (main.c:108-114, 129-135) without stalling the
 * timestep: the interior rows are staged device-to-device on the timestep
 * stream (so the next step may overwrite the field at once), copied from the
 * staging block to page-locked host memory on a side stream, and a writer
 * thread waits for that copy and writes <name><tt>.dat (the interior as
 * little-endian doubles, row by row) and <name><tt>.bov (its VisIt header).
 * kDumpSlots dumps may be in flight; a further call waits on the host for the
 * oldest to be written.  write_all_ranks_flush() waits for every pending dump
 * (it also runs at exit). */

enum { kDumpSlots = 2 };
enum { kSlotFree = 0, kSlotClaimed = 1, kSlotQueued = 2 };

struct DumpSlot {
  int state;               /* kSlotFree, kSlotClaimed or kSlotQueued */
  int device;
  double* d_stage;         /* interior block on the device */
  double* h_buf;           /* page-locked host copy */
  size_t cap;              /* doubles either buffer holds */
  size_t w, h;             /* interior width and height */
  cudaEvent_t staged, copied;
  char dat[256], bov[256], var[64];
  double time;
  unsigned long long seq;  /* order of the call */
};

static struct DumpSlot g_dump[kDumpSlots];
static pthread_mutex_t g_dump_lock = PTHREAD_MUTEX_INITIALIZER;
static pthread_cond_t g_dump_cond = PTHREAD_COND_INITIALIZER;
static pthread_t g_dump_thread;
static int g_dump_started = 0;
static cudaStream_t g_dump_stream = NULL;
static unsigned long long g_dump_seq = 0, g_dump_done = 0;

static void dump_write_files(struct DumpSlot* d) {
  FILE* fp = fopen(d->dat, "wb");
  if (!fp) TERMINATE("could not open %s\n", d->dat);
  if (fwrite(d->h_buf, sizeof(double), d->w * d->h, fp) != d->w * d->h) {
    TERMINATE("short write to %s\n", d->dat);
  }
  fclose(fp);
  fp = fopen(d->bov, "w");
  if (!fp) TERMINATE("could not open %s\n", d->bov);
  const char* base = strrchr(d->dat, '/');
  fprintf(fp, "TIME: %.12e\nDATA_FILE: %s\nDATA_SIZE: %zu %zu 1\n"
              "DATA_FORMAT: DOUBLE\nVARIABLE: %s\nDATA_ENDIAN: LITTLE\n"
              "CENTERING: zonal\nBRICK_ORIGIN: 0. 0. 0.\nBRICK_SIZE: %zu %zu 1\n",
          d->time, base ? base + 1 : d->dat, d->w, d->h, d->var, d->w, d->h);
  fclose(fp);
}

/* Writer thread: takes the queued slots in call order. */
static void* dump_writer(void* arg) {
  (void)arg;
  pthread_mutex_lock(&g_dump_lock);
  for (;;) {
    struct DumpSlot* next = NULL;
    while (!next) {
      for (int k = 0; k < kDumpSlots; ++k) {
        if (g_dump[k].state == kSlotQueued && g_dump[k].seq == g_dump_done) next = &g_dump[k];
      }
      if (!next) pthread_cond_wait(&g_dump_cond, &g_dump_lock);
    }
    pthread_mutex_unlock(&g_dump_lock);
    cuda_or_die(cudaSetDevice(next->device), "visit dump: cudaSetDevice");
    cuda_or_die(cudaEventSynchronize(next->copied), "visit dump copy");
    dump_write_files(next);
    pthread_mutex_lock(&g_dump_lock);
    next->state = kSlotFree;
    ++g_dump_done;
    pthread_cond_broadcast(&g_dump_cond);
  }
  return NULL;
}

void write_all_ranks_flush(void) {
  if (!g_dump_started) return;
  pthread_mutex_lock(&g_dump_lock);
  while (g_dump_done != g_dump_seq) pthread_cond_wait(&g_dump_cond, &g_dump_lock);
  pthread_mutex_unlock(&g_dump_lock);
}

void write_all_ranks_to_visit(const int global_nx, const int global_ny,
                              const int local_nx, const int local_ny,
                              const int pad, const int x_off, const int y_off,
                              const int rank, const int nranks,
                              int* neighbours, double* arr,
                              const char* arr_name, const int tt,
                              const double elapsed_sim_time) {
  (void)global_nx; (void)global_ny; (void)x_off; (void)y_off; (void)nranks;
  (void)neighbours;
  if (rank != MASTER) return;
  const size_t w = (size_t)(local_nx - 2 * pad), h = (size_t)(local_ny - 2 * pad);
  pthread_mutex_lock(&g_dump_lock);
  if (!g_dump_started) {
    cuda_or_die(cudaStreamCreateWithFlags(&g_dump_stream, cudaStreamNonBlocking),
                "visit dump: stream");
    if (pthread_create(&g_dump_thread, NULL, dump_writer, NULL) != 0) {
      TERMINATE("visit dump: could not start the writer thread\n");
    }
    pthread_detach(g_dump_thread);
    atexit(write_all_ranks_flush);
    g_dump_started = 1;
  }
  /* A free slot (the oldest dump is written first). */
  struct DumpSlot* d = NULL;
  while (!d) {
    for (int k = 0; k < kDumpSlots && !d; ++k) {
      if (g_dump[k].state == kSlotFree) d = &g_dump[k];
    }
    if (!d) pthread_cond_wait(&g_dump_cond, &g_dump_lock);
  }
  d->state = kSlotClaimed;
  pthread_mutex_unlock(&g_dump_lock);

  cuda_or_die(cudaGetDevice(&d->device), "visit dump: cudaGetDevice");
  if (d->cap < w * h) {
    if (d->d_stage) cudaFree(d->d_stage);
    if (d->h_buf) cudaFreeHost(d->h_buf);
    cuda_or_die(cudaMalloc((void**)&d->d_stage, w * h * sizeof(double)), "visit dump: cudaMalloc");
    cuda_or_die(cudaMallocHost((void**)&d->h_buf, w * h * sizeof(double)),
                "visit dump: cudaMallocHost");
    d->cap = w * h;
  }
  if (!d->staged) {
    cuda_or_die(cudaEventCreateWithFlags(&d->staged, cudaEventDisableTiming), "visit dump: event");
    cuda_or_die(cudaEventCreateWithFlags(&d->copied, cudaEventDisableTiming), "visit dump: event");
  }
  /* The interior rows, packed, on the stream that writes the field. */
  cudaStream_t s = (cudaStream_t)gb300_get_stream();
  cuda_or_die(cudaMemcpy2DAsync(d->d_stage, w * sizeof(double),
                                arr + (size_t)pad * local_nx + pad, (size_t)local_nx * sizeof(double),
                                w * sizeof(double), h, cudaMemcpyDeviceToDevice, s),
              "visit dump: staging copy");
  cuda_or_die(cudaEventRecord(d->staged, s), "visit dump: event");
  cuda_or_die(cudaStreamWaitEvent(g_dump_stream, d->staged, 0), "visit dump: wait");
  cuda_or_die(cudaMemcpyAsync(d->h_buf, d->d_stage, w * h * sizeof(double),
                              cudaMemcpyDeviceToHost, g_dump_stream),
              "visit dump: host copy");
  cuda_or_die(cudaEventRecord(d->copied, g_dump_stream), "visit dump: event");
  d->w = w;
  d->h = h;
  d->time = elapsed_sim_time;
  snprintf(d->dat, sizeof(d->dat), "%s%d.dat", arr_name, tt);
  snprintf(d->bov, sizeof(d->bov), "%s%d.bov", arr_name, tt);
  snprintf(d->var, sizeof(d->var), "%s", arr_name);
  pthread_mutex_lock(&g_dump_lock);
  d->seq = g_dump_seq++;
  d->state = kSlotQueued;
  pthread_cond_broadcast(&g_dump_cond);
  pthread_mutex_unlock(&g_dump_lock);
}
