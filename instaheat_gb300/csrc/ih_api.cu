// ih_api.cu -- the extern "C" entry points of libinstaheat_gpu.so
// (declared in include/instaheat_gpu.h) and the context lifecycle.
#include <math.h>
#include <string.h>
#include <new>
#include "ih_internal.cuh"

namespace ih {

int check_launch(Ctx *c, const char *what) {
  c->launches += 1;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    c->err = std::string(what) + ": " + cudaGetErrorString(e);
    return IH_ERR_CUDA;
  }
  return IH_OK;
}

const char *kernel_kind_name(int k) {
  static const char *names[KK_COUNT] = {
      "k_fft_xy",       "k_fft_zr2c",    "k_fft_zc2r",       "k_fft_x_deriv4_inv",
      "k_fft_xy_rt",    "k_fft_x_tensor", "k_fft_z_rhs_fused", "k_update_h", "k_update_phi_psi", "k_filter_spectra",
      "k_lincomb",      "k_dopri_final", "k_gw_plane2d", "k_update_h_plane",
      "k_gw_tt_plane", "k_update_h_tt"};
  return (k >= 0 && k < KK_COUNT) ? names[k] : "unknown";
}

int kernel_kind_class(int k) {
  if (k == KK_GW_PLANE || k == KK_GW_TT_PLANE) return 0;
  if (k == KK_UPDATE_H_PLANE || k == KK_UPDATE_H_TT) return 1;
  if (k <= KK_Z_RHS_FUSED) return 0;
  if (k <= KK_FILTER) return 1;
  return 2;
}

void prof_begin(Ctx *c, int kind) {
  if (!c->prof_on) return;
  cudaEvent_t e;
  cudaEventCreate(&e);
  cudaEventRecord(e, c->stream);
  c->timers[kind].ev.push_back(e);
}
void prof_end(Ctx *c, int kind, double bytes) {
  if (!c->prof_on) return;
  cudaEvent_t e;
  cudaEventCreate(&e);
  cudaEventRecord(e, c->stream);
  c->timers[kind].ev.push_back(e);
  c->timers[kind].launches += 1;
  c->timers[kind].bytes += bytes;
}

static bool pow2(int n) { return n >= 1 && (n & (n - 1)) == 0; }
// n = 2^a 3^b with a >= 1 (even: the real z transform halves nz)
static bool smooth23(int n) {
  if (n < 2 || n % 2) return false;
  while (n % 2 == 0) n /= 2;
  while (n % 3 == 0) n /= 3;
  return n == 1;
}

static int validate(const ih_params *p, std::string *why) {
  if (!p) {
    *why = "null parameters";
    return IH_ERR_ARG;
  }
  if (!smooth23(p->nx) || !smooth23(p->ny) || !smooth23(p->nz)) {
    *why = "grid sizes must be 2^a 3^b (a >= 1): powers of two, or with a radix-3 factor";
    return IH_ERR_ARG;
  }
  if (p->nx < p->ny || p->ny < p->nz) {
    *why = "order number of gridpoints Nx >= Ny >= Nz (setup.c:219-222)";
    return IH_ERR_ARG;
  }
  if (p->nz < 8) {
    *why = "the 3D GPU path needs nz >= 8";
    return IH_ERR_ARG;
  }
  if (p->nx > 512 || p->nz > 512) {
    *why = "grid too large for the FFT tiles (every axis <= 512)";
    return IH_ERR_ARG;
  }
  if (!(p->lx > 0 && p->ly > 0 && p->lz > 0)) {
    *why = "box lengths must be positive";
    return IH_ERR_ARG;
  }
  if (p->bins < 1) {
    *why = "POWER_SPECTRUM_BINS must be positive";
    return IH_ERR_ARG;
  }
  if (p->precision != IH_PREC_F64 && p->precision != IH_PREC_MIXED) {
    *why = "unknown precision";
    return IH_ERR_ARG;
  }
  return IH_OK;
}

static void make_geom(const ih_params *p, Geom *g) {
  g->nx = p->nx;
  g->ny = p->ny;
  g->nz = p->nz;
  g->h = p->nz / 2;
  g->mz = p->nz / 2 + 1;
  g->N = (long long)p->nx * p->ny * p->nz;
  g->M = (long long)p->nx * p->ny * g->mz;
  g->Next = 2 * g->M;
  g->Nf = 4 * g->N + 4 * g->Next;
  g->Ntot = g->Nf + 1;
  g->lx = p->lx;
  g->ly = p->ly;
  g->lz = p->lz;
  g->kxu = kTwoPi / p->lx;
  g->kyu = kTwoPi / p->ly;
  g->kzu = kTwoPi / p->lz;
  g->kx2 = kTwoPi * kTwoPi / (p->lx * p->lx);
  g->ky2 = kTwoPi * kTwoPi / (p->ly * p->ly);
  g->kz2 = kTwoPi * kTwoPi / (p->lz * p->lz);
  const double k2max = g->kx2 * (p->nx / 2) * (p->nx / 2) + g->ky2 * (p->ny / 2) * (p->ny / 2) +
                       g->kz2 * (p->nz / 2) * (p->nz / 2);
  g->kmax = sqrt(k2max);
  g->kxmax = (p->nx / 2) * g->kxu;
  g->kymax = (p->ny / 2) * g->kyu;
  g->kzmax = (p->nz / 2) * g->kzu;
  g->mass = p->mass;
  g->bins = p->bins;
  int l = 0;
  while ((1 << l) < g->mz) ++l;
  g->mz_shift = l;
  g->mz_magic = (unsigned)((((unsigned long long)1 << 32) * (((unsigned long long)1 << l) - g->mz)) /
                               g->mz + 1);
  g->logny = 0;
  while ((1 << g->logny) < g->ny) ++g->logny;
  g->pow2 = pow2(p->nx) && pow2(p->ny) && pow2(p->nz);
}

static int dmalloc(Ctx *c, void **p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    c->err = std::string("cudaMalloc(") + std::to_string(bytes) + "): " + cudaGetErrorString(e);
    return IH_ERR_ALLOC;
  }
  c->dev_bytes += bytes;
  return IH_OK;
}

static int alloc_vec(Ctx *c, Vec &v) {
  IH_TRY(dmalloc(c, &v.fl, c->tsize * c->g.Nf));
  IH_CUDA(c, cudaMemsetAsync(v.fl, 0, c->tsize * c->g.Nf, c->stream));
  IH_TRY(dmalloc(c, (void **)&v.sc, sizeof(double) * kSc));
  IH_CUDA(c, cudaMemsetAsync(v.sc, 0, sizeof(double) * kSc, c->stream));
  return IH_OK;
}

static void free_vec(Vec &v) {
  if (v.fl) cudaFree(v.fl);
  if (v.sc) cudaFree(v.sc);
  v.fl = nullptr;
  v.sc = nullptr;
}

static int create(const ih_params *p, Ctx *c) {
  c->p = *p;
  make_geom(p, &c->g);
  c->mixed = p->precision == IH_PREC_MIXED;
  c->tsize = c->mixed ? 4 : 8;
  c->noise_eta = c->mixed ? kDefaultNoiseEta : 0.0;
  IH_CUDA(c, cudaSetDevice(p->device));
  IH_CUDA(c, cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, p->device));
  IH_CUDA(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  const Geom &g = c->g;
  const size_t cs = 2 * c->tsize;  // complex element
  IH_TRY(fft_tables(c));
  void *specblk = nullptr;
  IH_TRY(dmalloc(c, &specblk, cs * (size_t)g.M * 7));
  for (int i = 0; i < 7; ++i) c->spec[i] = (char *)specblk + cs * (size_t)g.M * i;
  void *rblk = nullptr;
  IH_TRY(dmalloc(c, &rblk, c->tsize * (size_t)g.N * 4));
  for (int i = 0; i < 4; ++i) c->rbuf[i] = (char *)rblk + c->tsize * (size_t)g.N * i;
  IH_TRY(dmalloc(c, &c->mask, c->tsize * (size_t)g.M));
  if (!g.pow2) IH_TRY(dmalloc(c, &c->gscratch, c->tsize * (size_t)g.N * 6));
  // FP64 partial sums: the fused RHS pass writes 2 per tile of rows
  c->partials_cap = (long long)kMaxPartials * 8;
  if (2LL * g.nx * g.ny + 64 > c->partials_cap) c->partials_cap = 2LL * g.nx * g.ny + 64;
  IH_TRY(dmalloc(c, (void **)&c->partials, sizeof(double) * (size_t)c->partials_cap));
  IH_TRY(dmalloc(c, (void **)&c->rs, sizeof(RhsScalars)));
  IH_CUDA(c, cudaMemsetAsync(c->rs, 0, sizeof(RhsScalars), c->stream));
  IH_TRY(dmalloc(c, (void **)&c->diag, sizeof(double) * (4 * g.bins + 128)));
  IH_CUDA(c, cudaMemsetAsync(c->diag, 0, sizeof(double) * (4 * g.bins + 128), c->stream));
  IH_TRY(dmalloc(c, (void **)&c->waitflag, sizeof(int)));
  IH_CUDA(c, cudaMemsetAsync(c->waitflag, 0, sizeof(int), c->stream));
  if (c->mixed && p->enable_gw && g.nx == 256 && g.ny == 256 && g.nz == 256)
  {
    IH_TRY(dmalloc(c, &c->gwbuf, cs * (size_t)g.M * 6));
    IH_CUDA(c, cudaMemsetAsync(c->gwbuf, 0, cs * (size_t)g.M * 6, c->stream));
  }
  c->hpin_bytes = 4096;
  IH_CUDA(c, cudaMallocHost((void **)&c->hpin, c->hpin_bytes));
  IH_TRY(dmalloc(c, &c->stage_dev, sizeof(double) * (size_t)g.Ntot));
  IH_TRY(dmalloc(c, (void **)&c->dt_dev, sizeof(double)));
  IH_TRY(alloc_vec(c, c->y));
  IH_TRY(alloc_vec(c, c->ynew));
  IH_TRY(alloc_vec(c, c->ytmp));
  IH_TRY(alloc_vec(c, c->k[1]));
  IH_TRY(mask_init(c, c->mask));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  return IH_OK;
}

static void destroy(Ctx *c) {
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->tw_x) cudaFree(c->tw_x);
  if (c->tw_y) cudaFree(c->tw_y);
  if (c->tw_h) cudaFree(c->tw_h);
  if (c->tw_z) cudaFree(c->tw_z);
  if (c->spec[0]) cudaFree(c->spec[0]);
  if (c->rbuf[0]) cudaFree(c->rbuf[0]);
  if (c->gscratch) cudaFree(c->gscratch);
  if (c->mask) cudaFree(c->mask);
  if (c->partials) cudaFree(c->partials);
  if (c->rs) cudaFree(c->rs);
  if (c->diag) cudaFree(c->diag);
  if (c->waitflag) cudaFree(c->waitflag);
  if (c->gwbuf) cudaFree(c->gwbuf);
  if (c->hpin) cudaFreeHost(c->hpin);
  if (c->stage_dev) cudaFree(c->stage_dev);
  if (c->feat_dev) cudaFree(c->feat_dev);
  if (c->dt_dev) cudaFree(c->dt_dev);
  for (auto &gr : c->graphs)
    if (gr.exec) cudaGraphExecDestroy(gr.exec);
  c->graphs.clear();
  free_vec(c->y);
  free_vec(c->ynew);
  free_vec(c->ytmp);
  for (int j = 0; j < 13; ++j) free_vec(c->k[j]);
  for (int j = 0; j < 3; ++j) free_vec(c->kd[j]);
  free_vec(c->dense);
  for (auto &t : c->timers)
    for (auto e : t.ev) cudaEventDestroy(e);
  for (auto e : c->tev)
    if (e) cudaEventDestroy(e);
  if (c->stream) cudaStreamDestroy(c->stream);
}

static int upload_ref(Ctx *c, const double *host) {
  IH_CUDA(c, cudaMemcpyAsync(c->stage_dev, host, sizeof(double) * c->g.Ntot,
                             cudaMemcpyHostToDevice, c->stream));
  return IH_OK;
}
static int download_ref(Ctx *c, double *host) {
  IH_CUDA(c, cudaMemcpyAsync(host, c->stage_dev, sizeof(double) * c->g.Ntot,
                             cudaMemcpyDeviceToHost, c->stream));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  return IH_OK;
}

}  // namespace ih

using namespace ih;

struct ih_context {
  Ctx c;
};

#define CTX_CHECK(ctx)           \
  do {                           \
    if (!(ctx)) return IH_ERR_ARG; \
  } while (0)

extern "C" {

const char *ih_status_string(int s) {
  switch (s) {
    case IH_OK: return "ok";
    case IH_ERR_ARG: return "invalid argument";
    case IH_ERR_CUDA: return "CUDA error";
    case IH_ERR_ALLOC: return "allocation failed";
    case IH_ERR_STATE: return "call out of order";
    case IH_ERR_UNDERFLOW: return "step size underflow";
    case IH_ERR_NAN: return "non-finite value";
    case IH_ERR_TOO_LARGE: return "input larger than the fixed scratch of this entry point allows";
    default: return "unknown status";
  }
}

int ih_sizes(int nx, int ny, int nz, size_t *N, size_t *M, size_t *Next, size_t *Ntot) {
  if (nx < 1 || ny < 1 || nz < 2) return IH_ERR_ARG;
  size_t n = (size_t)nx * ny * nz, m = (size_t)nx * ny * (nz / 2 + 1);
  if (N) *N = n;
  if (M) *M = m;
  if (Next) *Next = 2 * m;
  if (Ntot) *Ntot = 4 * n + 4 * 2 * m + 1;
  return IH_OK;
}

int ih_create(const ih_params *p, ih_context **out) {
  if (!out) return IH_ERR_ARG;
  *out = nullptr;
  std::string why;
  int s = validate(p, &why);
  if (s != IH_OK) return s;
  ih_context *h = new (std::nothrow) ih_context();
  if (!h) return IH_ERR_ALLOC;
  s = create(p, &h->c);
  if (s != IH_OK) {
    destroy(&h->c);
    delete h;
    return s;
  }
  *out = h;
  return IH_OK;
}

void ih_destroy(ih_context *h) {
  if (!h) return;
  destroy(&h->c);
  delete h;
}

const char *ih_last_error(const ih_context *h) { return h ? h->c.err.c_str() : "null context"; }
size_t ih_device_bytes(const ih_context *h) { return h ? h->c.dev_bytes : 0; }
double ih_time(const ih_context *h) { return h ? h->c.t : 0.0; }
unsigned long long ih_calls_rhs(const ih_context *h) { return h ? h->c.calls_rhs : 0; }
unsigned long long ih_kernel_launches(const ih_context *h) { return h ? h->c.launches : 0; }

int ih_set_state(ih_context *h, const double *f, double t) {
  CTX_CHECK(h);
  if (!f) return IH_ERR_ARG;
  Ctx *c = &h->c;
  IH_TRY(upload_ref(c, f));
  IH_TRY(vec_from_ref(c, (const double *)c->stage_dev, c->y));
  c->t = t;
  c->have_state = 1;
  c->step_start_valid = 0;
  c->dense_ready = 0;
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  return IH_OK;
}

int ih_get_state(ih_context *h, double *f) {
  CTX_CHECK(h);
  if (!f) return IH_ERR_ARG;
  Ctx *c = &h->c;
  IH_TRY(vec_to_ref(c, c->y, (double *)c->stage_dev));
  return download_ref(c, f);
}

int ih_get_step_start_state(ih_context *h, double *f) {
  CTX_CHECK(h);
  if (!f) return IH_ERR_ARG;
  Ctx *c = &h->c;
  if (!c->step_start_valid) {
    c->err = "no step since the last mk_rhs or state upload";
    return IH_ERR_STATE;
  }
  IH_TRY(vec_to_ref(c, c->ynew, (double *)c->stage_dev));
  return download_ref(c, f);
}

int ih_set_dstate(ih_context *h, const double *df) {
  CTX_CHECK(h);
  if (!df) return IH_ERR_ARG;
  Ctx *c = &h->c;
  IH_TRY(upload_ref(c, df));
  IH_TRY(vec_from_ref(c, (const double *)c->stage_dev, c->k[1]));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  return IH_OK;
}

int ih_get_dstate(ih_context *h, double *df) {
  CTX_CHECK(h);
  if (!df) return IH_ERR_ARG;
  Ctx *c = &h->c;
  IH_TRY(vec_to_ref(c, c->k[1], (double *)c->stage_dev));
  return download_ref(c, df);
}

int ih_mk_rhs_dev(ih_context *h, double t, double *f_dev, double *result_dev, int filter,
                  int output) {
  CTX_CHECK(h);
  if (!f_dev || !result_dev) return IH_ERR_ARG;
  Ctx *c = &h->c;
  IH_TRY(vec_from_ref(c, f_dev, c->ytmp));
  c->step_start_valid = 0;
  c->dense_ready = 0;
  IH_TRY(rhs(c, t, c->ytmp, c->ynew, filter, output, nullptr));
  if (filter == 1 && c->p.enable_filter) IH_TRY(vec_to_ref(c, c->ytmp, f_dev));
  const Geom &g = c->g;
  if (c->p.enable_gw) {
    IH_TRY(vec_to_ref(c, c->ynew, result_dev));
  } else {
    // the reference leaves the tensor part of result untouched without GW
    IH_TRY(vec_to_ref(c, c->ynew, (double *)c->stage_dev));
    IH_CUDA(c, cudaMemcpyAsync(result_dev, c->stage_dev, sizeof(double) * 4 * g.N,
                               cudaMemcpyDeviceToDevice, c->stream));
    IH_CUDA(c, cudaMemcpyAsync(result_dev + g.Nf, (double *)c->stage_dev + g.Nf, sizeof(double),
                               cudaMemcpyDeviceToDevice, c->stream));
  }
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  return IH_OK;
}

int ih_mk_rhs_host(ih_context *h, double t, double *f, double *result, int filter, int output) {
  CTX_CHECK(h);
  if (!f || !result) return IH_ERR_ARG;
  Ctx *c = &h->c;
  const Geom &g = c->g;
  IH_TRY(upload_ref(c, f));
  IH_TRY(vec_from_ref(c, (const double *)c->stage_dev, c->ytmp));
  c->step_start_valid = 0;
  c->dense_ready = 0;
  IH_TRY(rhs(c, t, c->ytmp, c->ynew, filter, output, nullptr));
  if (filter == 1 && c->p.enable_filter) {
    IH_TRY(vec_to_ref(c, c->ytmp, (double *)c->stage_dev));
    IH_TRY(download_ref(c, f));
  }
  IH_TRY(vec_to_ref(c, c->ynew, (double *)c->stage_dev));
  if (c->p.enable_gw) return download_ref(c, result);
  IH_CUDA(c, cudaMemcpyAsync(result, c->stage_dev, sizeof(double) * 4 * g.N,
                             cudaMemcpyDeviceToHost, c->stream));
  IH_CUDA(c, cudaMemcpyAsync(result + g.Nf, (double *)c->stage_dev + g.Nf, sizeof(double),
                             cudaMemcpyDeviceToHost, c->stream));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  return IH_OK;
}

int ih_get_means(const ih_context *hc, double *rho_mean, double *pressure_mean) {
  if (!hc) return IH_ERR_ARG;
  ih_context *h = const_cast<ih_context *>(hc);
  Ctx *c = &h->c;
  IH_CUDA(c, cudaMemcpyAsync(&c->rs_host, c->rs, sizeof(RhsScalars), cudaMemcpyDeviceToHost,
                             c->stream));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  if (rho_mean) *rho_mean = c->rs_host.rho_mean;
  if (pressure_mean) *pressure_mean = c->rs_host.p_mean;
  return IH_OK;
}

int ih_get_field(ih_context *h, int which, double *out) {
  CTX_CHECK(h);
  if (!out) return IH_ERR_ARG;
  Ctx *c = &h->c;
  IH_TRY(get_field(c, which, (double *)c->stage_dev));
  IH_CUDA(c, cudaMemcpyAsync(out, c->stage_dev, sizeof(double) * c->g.N, cudaMemcpyDeviceToHost,
                             c->stream));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  return IH_OK;
}

int ih_get_output(ih_context *h, ih_output *out) {
  CTX_CHECK(h);
  if (!out) return IH_ERR_ARG;
  return read_output(&h->c, out);
}

int ih_mean_dev(ih_context *h, const double *f_dev, size_t n, double *out_dev) {
  CTX_CHECK(h);
  if (!f_dev || !out_dev || n == 0) return IH_ERR_ARG;
  Ctx *c = &h->c;
  IH_TRY(reduce_mean_f64(c, f_dev, (long long)n, out_dev));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  return IH_OK;
}

// mean / variance of a host array on the device; the results pass through
// diag slots 112-113
static int host_stats(ih_context *h, const double *f, size_t n, int var, double mean,
                      double *out) {
  CTX_CHECK(h);
  if (!f || !out || n == 0 || (var && n < 2)) return IH_ERR_ARG;
  Ctx *c = &h->c;
  if (n > c->g.Ntot) {
    c->err = "array longer than the staging buffer (Ntot doubles)";
    return IH_ERR_TOO_LARGE;
  }
  double *d = c->diag + 4 * c->g.bins + 112;
  IH_CUDA(c, cudaMemcpyAsync(c->stage_dev, f, sizeof(double) * n, cudaMemcpyHostToDevice,
                             c->stream));
  if (var) {
    IH_TRY(variance_f64(c, (const double *)c->stage_dev, (long long)n, mean, d));
  } else {
    IH_TRY(reduce_mean_f64(c, (const double *)c->stage_dev, (long long)n, d));
  }
  IH_CUDA(c, cudaMemcpyAsync(c->hpin, d, sizeof(double) * 2, cudaMemcpyDeviceToHost, c->stream));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  *out = var ? c->hpin[1] : c->hpin[0];
  return IH_OK;
}

int ih_mean_host(ih_context *h, const double *f_host, size_t n, double *out) {
  return host_stats(h, f_host, n, 0, 0.0, out);
}

int ih_variance_host(ih_context *h, double mean, const double *f_host, size_t n, double *out) {
  return host_stats(h, f_host, n, 1, mean, out);
}

int ih_autotune(ih_context *h) {
  CTX_CHECK(h);
  Ctx *c = &h->c;
  IH_TRY(fft_autotune(c));
  c->graph_epoch += 1;
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  return IH_OK;
}

const char *ih_autotune_report(const ih_context *h) {
  return h ? h->c.tune_report.c_str() : "";
}

int ih_fft_set_engine(ih_context *h, int pass, int engine) {
  CTX_CHECK(h);
  if (pass == 8) {  // plane-major tensor sources with the one-pass plane transforms
    if (engine < 0 || engine > 3) return IH_ERR_ARG;
    if (engine > 0 && !gw_plane_ok(&h->c)) {
      h->c.err = "the plane transforms apply to the mixed form at 256^3 with GW on";
      return IH_ERR_ARG;
    }
    h->c.gw_plane = engine;
    h->c.graph_epoch += 1;
    return IH_OK;
  }
  if (pass == 7) {  // kz slab width of the tensor sources' y/x passes
    if (engine < 0 || engine > 64 || engine % 8) return IH_ERR_ARG;
    h->c.gw_slab = engine;
    h->c.graph_epoch += 1;
    return IH_OK;
  }
  if (pass < 0 || pass > 6 || engine < 0 || engine >= FV_COUNT) return IH_ERR_ARG;
  if (pass == 2 && (engine == FV_THREESTEP || engine == FV_TWOSTEP_HALF_OCC)) return IH_ERR_ARG;
  if ((pass == 3 || pass == 4) && engine != FV_TWOSTEP && engine != FV_TWOSTEP_HALF)
    return IH_ERR_ARG;
  if (pass == 5 && engine > 1) return IH_ERR_ARG;
  if (pass == 6 && (engine > 2 || (engine == 2 && !h->c.mixed))) return IH_ERR_ARG;
  if (pass < 2) {
    h->c.xy_var[pass] = engine;
  } else if (pass == 2) {
    h->c.d4_var = engine;
  } else if (pass < 5) {
    h->c.rt_var[pass - 3] = engine;
  } else if (pass == 5) {
    h->c.tensor_fused = engine;
  } else {
    h->c.zwide = engine;
  }
  h->c.graph_epoch += 1;
  return IH_OK;
}

int ih_stage_fusion(ih_context *h, int on) {
  CTX_CHECK(h);
  h->c.stage_fusion = on ? 1 : 0;
  h->c.graph_epoch += 1;
  return IH_OK;
}

int ih_velocity_form(ih_context *h, int on) {
  CTX_CHECK(h);
  h->c.velocity_form = on ? 1 : 0;
  h->c.graph_epoch += 1;
  return IH_OK;
}

int ih_rhs_roundtrip(ih_context *h, int on) {
  CTX_CHECK(h);
  h->c.roundtrip = on ? 1 : 0;
  h->c.graph_epoch += 1;
  return IH_OK;
}

int ih_graphs_enable(ih_context *h, int on) {
  CTX_CHECK(h);
  h->c.graphs_on = on ? 1 : 0;
  return IH_OK;
}

int ih_fft_get_engine(const ih_context *h, int pass) {
  if (!h || pass < 0 || pass > 8) return -1;
  if (pass == 8) return h->c.gw_plane;
  if (pass == 7) return h->c.gw_slab;
  if (pass < 2) return h->c.xy_var[pass];
  if (pass == 5) return h->c.tensor_fused;
  if (pass == 6) return h->c.zwide;
  return pass == 2 ? h->c.d4_var : h->c.rt_var[pass - 3];
}

int ih_fft_host(ih_context *h, const double *in, double *out_c) {
  CTX_CHECK(h);
  if (!in || !out_c) return IH_ERR_ARG;
  Ctx *c = &h->c;
  const Geom &g = c->g;
  double *din = (double *)c->stage_dev, *dout = din + g.N;
  IH_CUDA(c, cudaMemcpyAsync(din, in, sizeof(double) * g.N, cudaMemcpyHostToDevice, c->stream));
  IH_TRY(fft_any(c, din, dout));
  IH_CUDA(c, cudaMemcpyAsync(out_c, dout, sizeof(double) * 2 * g.M, cudaMemcpyDeviceToHost,
                             c->stream));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  return IH_OK;
}

int ih_ifft_host(ih_context *h, const double *in_c, double *out) {
  CTX_CHECK(h);
  if (!in_c || !out) return IH_ERR_ARG;
  Ctx *c = &h->c;
  const Geom &g = c->g;
  double *din = (double *)c->stage_dev, *dout = din + 2 * g.M;
  IH_CUDA(c, cudaMemcpyAsync(din, in_c, sizeof(double) * 2 * g.M, cudaMemcpyHostToDevice,
                             c->stream));
  IH_TRY(ifft_any(c, din, dout));
  IH_CUDA(c, cudaMemcpyAsync(out, dout, sizeof(double) * g.N, cudaMemcpyDeviceToHost,
                             c->stream));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  return IH_OK;
}

int ih_ic_fluctuations(ih_context *h, uint64_t seed, double phi0, double dphi0, double a0,
                       double amp, double kcut) {
  CTX_CHECK(h);
  Ctx *c = &h->c;
  IH_TRY(ic_fluctuations(c, seed, phi0, dphi0, a0, amp, kcut));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  c->have_state = 1;
  c->dopri_ready = 0;
  return IH_OK;
}

int ih_initial_psi(ih_context *h) {
  CTX_CHECK(h);
  Ctx *c = &h->c;
  if (!c->have_state) {
    c->err = "no state";
    return IH_ERR_STATE;
  }
  IH_TRY(initial_psi(c));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  c->dopri_ready = 0;
  return IH_OK;
}

int ih_dopri853_init(ih_context *h, const ih_dopri_cfg *cfg, double t0, double dt0) {
  return ih_dopri853_init_ex(h, cfg, t0, dt0, 0);
}

int ih_dopri853_init_ex(ih_context *h, const ih_dopri_cfg *cfg, double t0, double dt0,
                        int want_output) {
  CTX_CHECK(h);
  if (!cfg || !(cfg->rtol >= 0) || !(cfg->atol >= 0) || !(dt0 > 0)) return IH_ERR_ARG;
  Ctx *c = &h->c;
  if (!c->have_state) {
    c->err = "no state";
    return IH_ERR_STATE;
  }
  IH_TRY(dopri_init(c, cfg, t0, dt0, want_output ? 1 : 0));
  c->graph_epoch += 1;  // the tolerances are baked into the captured try
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  return IH_OK;
}

int ih_dopri853_step(ih_context *h, double dt_try, int want_output, ih_step_info *info) {
  CTX_CHECK(h);
  if (!(dt_try > 0)) return IH_ERR_ARG;
  return dopri_step(&h->c, dt_try, want_output, info);
}

int ih_dopri853_run(ih_context *h, double tf, long max_steps, double *log, long log_cap,
                    long *n_steps) {
  CTX_CHECK(h);
  Ctx *c = &h->c;
  if (!c->dopri_ready) {
    c->err = "ih_dopri853_init has not been called";
    return IH_ERR_STATE;
  }
  // the run loop of dopri853.c:118-155 (I/O and wall-clock limits are the
  // caller's; the C99 drop-in layer adds them)
  double dt = c->dt_next;
  long accepted = 0;
  int status = IH_OK;
  for (c->n_stp = 0;; ++c->n_stp) {
    if (c->t + dt * 1.0001 > tf) dt = tf - c->t;
    ih_step_info info;
    status = dopri_step(c, dt, 0, &info);
    if (status != IH_OK) break;
    ++accepted;
    if (info.dt_did == dt) ++c->n_ok;
    else ++c->n_bad;
    if (log && c->n_stp < log_cap) {
      log[4 * c->n_stp] = info.t;
      log[4 * c->n_stp + 1] = info.dt_did;
      log[4 * c->n_stp + 2] = info.err;
      log[4 * c->n_stp + 3] = info.tries;
    }
    if (c->t >= tf) break;
    if (c->n_stp + 1 >= max_steps) break;
    if (fabs(c->dt_next) <= c->cfg.dt_min) {
      // the reference prints "Stepsize underflow" and ends the run
      // (dopri853.c:150-153); here the caller sees the status
      c->err = "proposed step size at or below MINIMAL_DELTA_T";
      status = IH_ERR_UNDERFLOW;
      break;
    }
    dt = c->dt_next;
  }
  if (n_steps) *n_steps = accepted;
  return status;
}

int ih_dopri853_counters(const ih_context *h, double *dt_next, long *n_ok, long *n_bad,
                         long *n_tries) {
  if (!h) return IH_ERR_ARG;
  const Ctx *c = &h->c;
  if (dt_next) *dt_next = c->dt_next;
  if (n_ok) *n_ok = c->n_ok;
  if (n_bad) *n_bad = c->n_bad;
  if (n_tries) *n_tries = c->n_tries;
  return IH_OK;
}

int ih_dopri853_tableau(double *cc, double *a, double *b, double *bhh, double *er) {
  dopri_tableau(cc, a, b, bhh, er);
  return IH_OK;
}

int ih_dopri853_dense_tableau(double *ad, double *d) {
  dopri_dense_tableau(ad, d);
  return IH_OK;
}

int ih_dopri853_dense(ih_context *h, double t_out, int want_output, double *field_out) {
  CTX_CHECK(h);
  Ctx *c = &h->c;
  IH_TRY(dopri_dense(c, t_out, want_output ? 1 : 0));
  if (field_out) {
    IH_TRY(vec_to_ref(c, c->dense, (double *)c->stage_dev));
    IH_TRY(download_ref(c, field_out));
  }
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  return IH_OK;
}

int ih_rk4_step(ih_context *h, double dt, int want_output) {
  CTX_CHECK(h);
  Ctx *c = &h->c;
  if (!c->have_state) {
    c->err = "no state";
    return IH_ERR_STATE;
  }
  IH_TRY(rk4_step(c, dt, want_output));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  return IH_OK;
}

int ih_sync(ih_context *h) {
  CTX_CHECK(h);
  Ctx *c = &h->c;
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  return IH_OK;
}

int ih_profile_enable(ih_context *h, int on) {
  CTX_CHECK(h);
  Ctx *c = &h->c;
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  for (auto &t : c->timers) {
    for (auto e : t.ev) cudaEventDestroy(e);
    t.ev.clear();
    t.bytes = 0.0;
    t.launches = 0;
  }
  c->prof_on = on;
  return IH_OK;
}

static double timer_ms(Timer &t) {
  double total = 0.0;
  for (size_t i = 0; i + 1 < t.ev.size(); i += 2) {
    float f = 0.f;
    cudaEventElapsedTime(&f, t.ev[i], t.ev[i + 1]);
    total += f;
  }
  return total;
}

int ih_profile_read(ih_context *h, int cls, double *ms, long *launches) {
  CTX_CHECK(h);
  if (cls < 0 || cls > 2) return IH_ERR_ARG;
  Ctx *c = &h->c;
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  double total = 0.0;
  long n = 0;
  for (int k = 0; k < KK_COUNT; ++k) {
    if (kernel_kind_class(k) != cls) continue;
    total += timer_ms(c->timers[k]);
    n += c->timers[k].launches;
  }
  if (ms) *ms = total;
  if (launches) *launches = n;
  return IH_OK;
}

int ih_profile_kernel(ih_context *h, int kind, double *ms, long *launches, double *bytes) {
  CTX_CHECK(h);
  if (kind < 0 || kind >= KK_COUNT) return IH_ERR_ARG;
  Ctx *c = &h->c;
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  Timer &t = c->timers[kind];
  if (ms) *ms = timer_ms(t);
  if (launches) *launches = t.launches;
  if (bytes) *bytes = t.bytes;
  return IH_OK;
}

const char *ih_profile_kernel_name(int kind) { return kernel_kind_name(kind); }
int ih_profile_kernel_count(void) { return KK_COUNT; }

int ih_timer_start(ih_context *h) {
  CTX_CHECK(h);
  Ctx *c = &h->c;
  for (int i = 0; i < 2; ++i)
    if (!c->tev[i]) IH_CUDA(c, cudaEventCreate(&c->tev[i]));
  IH_CUDA(c, cudaEventRecord(c->tev[0], c->stream));
  return IH_OK;
}

int ih_timer_stop(ih_context *h, double *ms) {
  CTX_CHECK(h);
  Ctx *c = &h->c;
  if (!c->tev[0]) return IH_ERR_STATE;
  IH_CUDA(c, cudaEventRecord(c->tev[1], c->stream));
  IH_CUDA(c, cudaEventSynchronize(c->tev[1]));
  float f = 0.f;
  IH_CUDA(c, cudaEventElapsedTime(&f, c->tev[0], c->tev[1]));
  if (ms) *ms = f;
  return IH_OK;
}

int ih_host_alloc(size_t bytes, void **out) {
  if (!out) return IH_ERR_ARG;
  *out = nullptr;
  if (cudaMallocHost(out, bytes) != cudaSuccess) return IH_ERR_ALLOC;
  return IH_OK;
}

int ih_host_free(void *p) {
  if (p && cudaFreeHost(p) != cudaSuccess) return IH_ERR_CUDA;
  return IH_OK;
}

int ih_step_features(ih_context *h, float *out12) {
  CTX_CHECK(h);
  if (!out12) return IH_ERR_ARG;
  return step_features(&h->c, out12);
}

int ih_dopri853_set_proposer(ih_context *h, ih_mlp *m) {
  CTX_CHECK(h);
  Ctx *c = &h->c;
  if (m && !c->feat_dev) IH_TRY(dmalloc(c, (void **)&c->feat_dev, sizeof(float) * 16));
  c->proposer = m;
  return IH_OK;
}

int ih_prepare_output(ih_context *h) {
  CTX_CHECK(h);
  Ctx *c = &h->c;
  if (!c->have_state) {
    c->err = "no state";
    return IH_ERR_STATE;
  }
  IH_TRY(rhs(c, c->t, c->y, c->k[1], 1, 1, nullptr));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  return IH_OK;
}

int ih_dopri853_diag_enable(ih_context *h, int on) {
  CTX_CHECK(h);
  h->c.err_diag = on ? 1 : 0;
  return IH_OK;
}

int ih_dopri853_error_breakdown(ih_context *h, double *out12) {
  CTX_CHECK(h);
  if (!out12) return IH_ERR_ARG;
  Ctx *c = &h->c;
  if (!c->err_diag) return IH_ERR_STATE;
  IH_CUDA(c, cudaMemcpyAsync(out12, c->diag + 4 * c->g.bins + 72, sizeof(double) * 12,
                             cudaMemcpyDeviceToHost, c->stream));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  return IH_OK;
}

int ih_dopri853_set_noise_floor(ih_context *h, double eta) {
  CTX_CHECK(h);
  if (!(eta >= 0.0)) return IH_ERR_ARG;
  h->c.noise_eta = eta;
  h->c.graph_epoch += 1;
  return IH_OK;
}

// ---------------------------------------------------------------------------
// ensembles: member contexts stepped together
struct ih_ensemble {
  std::vector<ih_context *> m;
  std::string err;
};

int ih_ensemble_create(const ih_params *members, int count, ih_ensemble **out) {
  if (!out || !members || count < 1) return IH_ERR_ARG;
  *out = nullptr;
  ih_ensemble *e = new (std::nothrow) ih_ensemble();
  if (!e) return IH_ERR_ALLOC;
  for (int i = 0; i < count; ++i) {
    ih_context *h = nullptr;
    const int s = ih_create(&members[i], &h);
    if (s != IH_OK) {
      for (auto x : e->m) ih_destroy(x);
      delete e;
      return s;
    }
    e->m.push_back(h);
  }
  *out = e;
  return IH_OK;
}

void ih_ensemble_destroy(ih_ensemble *e) {
  if (!e) return;
  for (auto x : e->m) ih_destroy(x);
  delete e;
}

const char *ih_ensemble_last_error(const ih_ensemble *e) { return e ? e->err.c_str() : "null ensemble"; }
int ih_ensemble_size(const ih_ensemble *e) { return e ? (int)e->m.size() : 0; }
ih_context *ih_ensemble_member(ih_ensemble *e, int i) {
  return (e && i >= 0 && i < (int)e->m.size()) ? e->m[i] : nullptr;
}

static int ens_fail(ih_ensemble *e, int i, int s) {
  e->err = "member " + std::to_string(i) + ": " + ih_last_error(e->m[i]);
  return s;
}

int ih_ensemble_autotune(ih_ensemble *e) {
  if (!e) return IH_ERR_ARG;
  // one tuning per distinct grid and precision, copied to the members alike
  for (size_t i = 0; i < e->m.size(); ++i) {
    Ctx *c = &e->m[i]->c;
    const Ctx *twin = nullptr;
    for (size_t j = 0; j < i; ++j) {
      const Ctx *d = &e->m[j]->c;
      if (d->g.nx == c->g.nx && d->g.ny == c->g.ny && d->g.nz == c->g.nz && d->mixed == c->mixed &&
          d->p.device == c->p.device)
        twin = d;
    }
    if (twin) {
      c->xy_var[0] = twin->xy_var[0];
      c->xy_var[1] = twin->xy_var[1];
      c->d4_var = twin->d4_var;
      c->rt_var[0] = twin->rt_var[0];
      c->rt_var[1] = twin->rt_var[1];
      c->tensor_fused = twin->tensor_fused;
      c->zwide = twin->zwide;
      c->gw_slab = twin->gw_slab;
      c->velocity_form = twin->velocity_form;
      c->tune_report = twin->tune_report;
      c->graph_epoch += 1;
    } else {
      const int s = ih_autotune(e->m[i]);
      if (s != IH_OK) return ens_fail(e, (int)i, s);
    }
  }
  return IH_OK;
}

int ih_ensemble_dopri_init(ih_ensemble *e, const ih_dopri_cfg *cfg, double t0, double dt0) {
  if (!e) return IH_ERR_ARG;
  for (size_t i = 0; i < e->m.size(); ++i) {
    const int s = ih_dopri853_init(e->m[i], cfg, t0, dt0);
    if (s != IH_OK) return ens_fail(e, (int)i, s);
  }
  return IH_OK;
}

int ih_ensemble_run(ih_ensemble *e, double tf, long max_rounds, long *rounds_out,
                    long *steps_out) {
  if (!e) return IH_ERR_ARG;
  const size_t n = e->m.size();
  // per member: the run loop of dopri853.c:118-155 (as ih_dopri853_run), one
  // try per round; all members' tries of a round are queued before any is
  // waited for, so they run concurrently on the members' streams
  std::vector<double> dt(n), dt_step(n);
  std::vector<int> active(n), fresh(n, 1), tries(n, 0);
  for (size_t i = 0; i < n; ++i) {
    Ctx *c = &e->m[i]->c;
    if (!c->dopri_ready) {
      e->err = "member " + std::to_string(i) + ": ih_dopri853_init has not been called";
      return IH_ERR_STATE;
    }
    dt[i] = c->dt_next;
    active[i] = c->t < tf;
  }
  long rounds = 0, steps = 0;
  for (; rounds < max_rounds; ++rounds) {
    bool any = false;
    for (size_t i = 0; i < n; ++i) {
      if (!active[i]) continue;
      any = true;
      Ctx *c = &e->m[i]->c;
      if (fresh[i]) {
        if (c->t + dt[i] * 1.0001 > tf) dt[i] = tf - c->t;
        dt_step[i] = dt[i];
        fresh[i] = 0;
        tries[i] = 0;
      }
      const int s = try_enqueue(c, dt[i]);
      if (s != IH_OK) return ens_fail(e, (int)i, s);
    }
    if (!any) break;
    for (size_t i = 0; i < n; ++i) {
      if (!active[i]) continue;
      Ctx *c = &e->m[i]->c;
      double err, rho_mean;
      int nonfinite;
      int s = try_collect(c, &err, &rho_mean, &nonfinite);
      if (s != IH_OK) return ens_fail(e, (int)i, s);
      ++tries[i];
      const int o = try_outcome(c, err, rho_mean, nonfinite, &dt[i]);
      if (o < 0) return ens_fail(e, (int)i, -o);
      if (o == 0) continue;  // retry with the reduced dt next round
      ih_step_info info;
      s = step_accept(c, dt[i], err, rho_mean, 0, tries[i], &info);
      if (s != IH_OK) return ens_fail(e, (int)i, s);
      ++steps;
      if (info.dt_did == dt_step[i]) {
        ++c->n_ok;
      } else {
        ++c->n_bad;
      }
      ++c->n_stp;
      fresh[i] = 1;
      if (c->t >= tf || fabs(c->dt_next) <= c->cfg.dt_min || (double)c->n_stp >= c->cfg.max_steps) {
        active[i] = 0;
      } else {
        dt[i] = c->dt_next;
      }
    }
  }
  for (size_t i = 0; i < n; ++i) {
    const cudaError_t ce = cudaStreamSynchronize(e->m[i]->c.stream);
    if (ce != cudaSuccess) {
      e->err = std::string("member stream: ") + cudaGetErrorString(ce);
      return IH_ERR_CUDA;
    }
  }
  if (rounds_out) *rounds_out = rounds;
  if (steps_out) *steps_out = steps;
  return IH_OK;
}

}  // extern "C"
