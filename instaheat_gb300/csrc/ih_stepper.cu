// ih_stepper.cu -- DOPRI853 (src/dopri853.c) and RK4 (src/rk4.c) on GB300.
//
// The state and all stage vectors stay on the device.  Per try the host
// launches 11 stage combinations + 11 RHS evaluations and one fused kernel
// that forms field_new and both embedded error sums (dopri853.c:438-486),
// then reads back 4 doubles (error sums, <rho>, NaN flag) and runs the
// reference's controller (dopri853.c:505-540) on the host.  Accepted steps
// swap buffer pointers instead of copying field_new/dfield_new
// (dopri853.c:301-305).
//
// Stage combinations and the final combination are bandwidth kernels over
// Nf = 4N + 4Next elements: 16-byte vector loads (float4 / double2), grid
// sized to a multiple of the 152 SMs, FP64 homogeneous parts handled by one
// thread.
#include <float.h>
#include <math.h>
#include <string.h>
#include <mutex>
#include "ih_internal.cuh"

namespace ih {

// ---------------------------------------------------------------------------
// Dormand-Prince 8(5,3) coefficients as published by Hairer, Norsett and
// Wanner (code DOP853); the reference takes the same numbers from Numerical
// Recipes (src/dopri853_constants.c).  Stages 1..12; A[i][j] = a_{i+1,j+1}.
static double DA[12][12], DB[12], DE3[12], DBHH[3];
static const double DC[12] = {0.0,
                              0.526001519587677318785587544488e-01,
                              0.789002279381515978178381316732e-01,
                              0.118350341907227396726757197510e+00,
                              0.281649658092772603273242802490e+00,
                              0.333333333333333333333333333333e+00,
                              0.25e+00,
                              0.307692307692307692307692307692e+00,
                              0.651282051282051282051282051282e+00,
                              0.6e+00,
                              0.857142857142857142857142857142e+00,
                              1.0};
// Dense output (the same authors' continuous extension; the reference
// declares these in src/dopri853_constants.c:23-25, 98-173 and never uses
// them): DAD[r] = the input of stage 14 + r over stages 1..16 (stage 13 =
// f(field_new)), DDN[i] = the weights d(4+i) over stages 1..16.
static double DAD[3][16], DDN[4][16];
static int tableau_ready = 0;

static void tableau_init() {
  if (tableau_ready) return;
  memset(DA, 0, sizeof DA);
  memset(DB, 0, sizeof DB);
  memset(DE3, 0, sizeof DE3);
  double(*A)[12] = DA;
  A[1][0] = 5.26001519587677318785587544488e-2;
  A[2][0] = 1.97250569845378994544595329183e-2;
  A[2][1] = 5.91751709536136983633785987549e-2;
  A[3][0] = 2.95875854768068491816892993775e-2;
  A[3][2] = 8.87627564304205475450678981324e-2;
  A[4][0] = 2.41365134159266685502369798665e-1;
  A[4][2] = -8.84549479328286085344864962717e-1;
  A[4][3] = 9.24834003261792003115737966543e-1;
  A[5][0] = 3.7037037037037037037037037037e-2;
  A[5][3] = 1.70828608729473871279604482173e-1;
  A[5][4] = 1.25467687566822425016691814123e-1;
  A[6][0] = 3.7109375e-2;
  A[6][3] = 1.70252211019544039314978060272e-1;
  A[6][4] = 6.02165389804559606850219397283e-2;
  A[6][5] = -1.7578125e-2;
  A[7][0] = 3.70920001185047927108779319836e-2;
  A[7][3] = 1.70383925712239993810214054705e-1;
  A[7][4] = 1.07262030446373284651809199168e-1;
  A[7][5] = -1.53194377486244017527936158236e-2;
  A[7][6] = 8.27378916381402288758473766002e-3;
  A[8][0] = 6.24110958716075717114429577812e-1;
  A[8][3] = -3.36089262944694129406857109825e0;
  A[8][4] = -8.68219346841726006818189891453e-1;
  A[8][5] = 2.75920996994467083049415600797e1;
  A[8][6] = 2.01540675504778934086186788979e1;
  A[8][7] = -4.34898841810699588477366255144e1;
  A[9][0] = 4.77662536438264365890433908527e-1;
  A[9][3] = -2.48811461997166764192642586468e0;
  A[9][4] = -5.90290826836842996371446475743e-1;
  A[9][5] = 2.12300514481811942347288949897e1;
  A[9][6] = 1.52792336328824235832596922938e1;
  A[9][7] = -3.32882109689848629194453265587e1;
  A[9][8] = -2.03312017085086261358222928593e-2;
  A[10][0] = -9.3714243008598732571704021658e-1;
  A[10][3] = 5.18637242884406370830023853209e0;
  A[10][4] = 1.09143734899672957818500254654e0;
  A[10][5] = -8.14978701074692612513997267357e0;
  A[10][6] = -1.85200656599969598641566180701e1;
  A[10][7] = 2.27394870993505042818970056734e1;
  A[10][8] = 2.49360555267965238987089396762e0;
  A[10][9] = -3.0467644718982195003823669022e0;
  A[11][0] = 2.27331014751653820792359768449e0;
  A[11][3] = -1.05344954667372501984066689879e1;
  A[11][4] = -2.00087205822486249909675718444e0;
  A[11][5] = -1.79589318631187989172765950534e1;
  A[11][6] = 2.79488845294199600508499808837e1;
  A[11][7] = -2.85899827713502369474065508674e0;
  A[11][8] = -8.87285693353062954433549289258e0;
  A[11][9] = 1.23605671757943030647266201528e1;
  A[11][10] = 6.43392746015763530355970484046e-1;
  DB[0] = 5.42937341165687622380535766363e-2;
  DB[5] = 4.45031289275240888144113950566e0;
  DB[6] = 1.89151789931450038304281599044e0;
  DB[7] = -5.8012039600105847814672114227e0;
  DB[8] = 3.1116436695781989440891606237e-1;
  DB[9] = -1.52160949662516078556178806805e-1;
  DB[10] = 2.01365400804030348374776537501e-1;
  DB[11] = 4.47106157277725905176885569043e-2;
  DBHH[0] = 0.244094488188976377952755905512e+00;
  DBHH[1] = 0.733846688281611857341361741547e+00;
  DBHH[2] = 0.220588235294117647058823529412e-01;
  DE3[0] = 0.1312004499419488073250102996e-01;
  DE3[5] = -0.1225156446376204440720569753e+01;
  DE3[6] = -0.4957589496572501915214079952e+00;
  DE3[7] = 0.1664377182454986536961530415e+01;
  DE3[8] = -0.3503288487499736816886487290e+00;
  DE3[9] = 0.3341791187130174790297318841e+00;
  DE3[10] = 0.8192320648511571246570742613e-01;
  DE3[11] = -0.2235530786388629525884427845e-01;
  memset(DAD, 0, sizeof DAD);
  memset(DDN, 0, sizeof DDN);
  double(*AD)[16] = DAD;
  double(*DD)[16] = DDN;
  AD[0][0] = 5.61675022830479523392909219681e-2;
  AD[0][6] = 2.53500210216624811088794765333e-1;
  AD[0][7] = -2.46239037470802489917441475441e-1;
  AD[0][8] = -1.24191423263816360469010140626e-1;
  AD[0][9] = 1.5329179827876569731206322685e-1;
  AD[0][10] = 8.20105229563468988491666602057e-3;
  AD[0][11] = 7.56789766054569976138603589584e-3;
  AD[0][12] = -8.298e-3;
  AD[1][0] = 3.18346481635021405060768473261e-2;
  AD[1][5] = 2.83009096723667755288322961402e-2;
  AD[1][6] = 5.35419883074385676223797384372e-2;
  AD[1][7] = -5.49237485713909884646569340306e-2;
  AD[1][10] = -1.08347328697249322858509316994e-4;
  AD[1][11] = 3.82571090835658412954920192323e-4;
  AD[1][12] = -3.40465008687404560802977114492e-4;
  AD[1][13] = 1.41312443674632500278074618366e-1;
  AD[2][0] = -4.28896301583791923408573538692e-1;
  AD[2][5] = -4.69762141536116384314449447206e0;
  AD[2][6] = 7.68342119606259904184240953878e0;
  AD[2][7] = 4.06898981839711007970213554331e0;
  AD[2][8] = 3.56727187455281109270669543021e-1;
  AD[2][12] = -1.39902416515901462129418009734e-3;
  AD[2][13] = 2.9475147891527723389556272149e0;
  AD[2][14] = -9.15095847217987001081870187138e0;
  DD[0][0] = -0.84289382761090128651353491142e+01;
  DD[0][5] = 0.56671495351937776962531783590e+00;
  DD[0][6] = -0.30689499459498916912797304727e+01;
  DD[0][7] = 0.23846676565120698287728149680e+01;
  DD[0][8] = 0.21170345824450282767155149946e+01;
  DD[0][9] = -0.87139158377797299206789907490e+00;
  DD[0][10] = 0.22404374302607882758541771650e+01;
  DD[0][11] = 0.63157877876946881815570249290e+00;
  DD[0][12] = -0.88990336451333310820698117400e-01;
  DD[0][13] = 0.18148505520854727256656404962e+02;
  DD[0][14] = -0.91946323924783554000451984436e+01;
  DD[0][15] = -0.44360363875948939664310572000e+01;
  DD[1][0] = 0.10427508642579134603413151009e+02;
  DD[1][5] = 0.24228349177525818288430175319e+03;
  DD[1][6] = 0.16520045171727028198505394887e+03;
  DD[1][7] = -0.37454675472269020279518312152e+03;
  DD[1][8] = -0.22113666853125306036270938578e+02;
  DD[1][9] = 0.77334326684722638389603898808e+01;
  DD[1][10] = -0.30674084731089398182061213626e+02;
  DD[1][11] = -0.93321305264302278729567221706e+01;
  DD[1][12] = 0.15697238121770843886131091075e+02;
  DD[1][13] = -0.31139403219565177677282850411e+02;
  DD[1][14] = -0.93529243588444783865713862664e+01;
  DD[1][15] = 0.35816841486394083752465898540e+02;
  DD[2][0] = 0.19985053242002433820987653617e+02;
  DD[2][5] = -0.38703730874935176555105901742e+03;
  DD[2][6] = -0.18917813819516756882830838328e+03;
  DD[2][7] = 0.52780815920542364900561016686e+03;
  DD[2][8] = -0.11573902539959630126141871134e+02;
  DD[2][9] = 0.68812326946963000169666922661e+01;
  DD[2][10] = -0.10006050966910838403183860980e+01;
  DD[2][11] = 0.77771377980534432092869265740e+00;
  DD[2][12] = -0.27782057523535084065932004339e+01;
  DD[2][13] = -0.60196695231264120758267380846e+02;
  DD[2][14] = 0.84320405506677161018159903784e+02;
  DD[2][15] = 0.11992291136182789328035130030e+02;
  DD[3][0] = -0.25693933462703749003312586129e+02;
  DD[3][5] = -0.15418974869023643374053993627e+03;
  DD[3][6] = -0.23152937917604549567536039109e+03;
  DD[3][7] = 0.35763911791061412378285349910e+03;
  DD[3][8] = 0.93405324183624310003907691704e+02;
  DD[3][9] = -0.37458323136451633156875139351e+02;
  DD[3][10] = 0.10409964950896230045147246184e+03;
  DD[3][11] = 0.29840293426660503123344363579e+02;
  DD[3][12] = -0.43533456590011143754432175058e+02;
  DD[3][13] = 0.96324553959188282948394950600e+02;
  DD[3][14] = -0.39177261675615439165231486172e+02;
  DD[3][15] = -0.14972683625798562581422125276e+03;
  tableau_ready = 1;
}

void dopri_dense_tableau(double *ad, double *d) {
  tableau_init();
  if (ad) memcpy(ad, DAD, sizeof DAD);
  if (d) memcpy(d, DDN, sizeof DDN);
}

void dopri_tableau(double *cc, double *a, double *b, double *bhh, double *er) {
  tableau_init();
  if (cc) memcpy(cc, DC, sizeof DC);
  if (a) memcpy(a, DA, sizeof DA);
  if (b) memcpy(b, DB, sizeof DB);
  if (bhh) memcpy(bhh, DBHH, sizeof DBHH);
  if (er) memcpy(er, DE3, sizeof DE3);
}

// ---------------------------------------------------------------------------
struct LinArgs {
  const void *in[kMaxTerms];
  const double *insc[kMaxTerms];
  double coef[kMaxTerms];
  int n;
  double scale;            // out = base + scale * sum coef_j in_j
  const double *scale_dev;  // if set, the scale is read from device memory
};

template <typename T> struct Vec4;
template <> struct Vec4<float> {
  using type = float4;
  static constexpr int W = 4;
};
template <> struct Vec4<double> {
  using type = double2;
  static constexpr int W = 2;
};

template <typename T>
__device__ __forceinline__ void vload(const T *p, T *v) {
  if constexpr (sizeof(T) == 4) {
    float4 q = *reinterpret_cast<const float4 *>(p);
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
  } else {
    double2 q = *reinterpret_cast<const double2 *>(p);
    v[0] = q.x; v[1] = q.y;
  }
}
template <typename T>
__device__ __forceinline__ void vstore(T *p, const T *v) {
  if constexpr (sizeof(T) == 4) {
    *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
  } else {
    *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]);
  }
}

// y_stage = y + dt * sum_j a_sj k_j (dopri853.c:340-436, rk4.c:131-150)
template <typename T>
__global__ void k_lincomb(const T *__restrict__ base, const double *basesc, T *__restrict__ out,
                          double *outsc, LinArgs args, long long nf) {
  constexpr int W = Vec4<T>::W;
  const long long nv = nf / W;
  T cf[kMaxTerms];
#pragma unroll
  for (int j = 0; j < kMaxTerms; ++j) cf[j] = (T)args.coef[j];
  const double scd = args.scale_dev ? *args.scale_dev : args.scale;
  const T sc = (T)scd;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv;
       v += (long long)gridDim.x * blockDim.x) {
    T acc[W], x[W];
#pragma unroll
    for (int w = 0; w < W; ++w) acc[w] = 0;
#pragma unroll
    for (int j = 0; j < kMaxTerms; ++j) {
      if (j < args.n) {
        vload<T>((const T *)args.in[j] + v * W, x);
#pragma unroll
        for (int w = 0; w < W; ++w) acc[w] += cf[j] * x[w];
      }
    }
    vload<T>(base + v * W, x);
#pragma unroll
    for (int w = 0; w < W; ++w) x[w] = x[w] + sc * acc[w];
    vstore<T>(out + v * W, x);
  }
  if (blockIdx.x == 0 && threadIdx.x < 5) {
    const int s = threadIdx.x;
    double acc = 0.0;
    for (int j = 0; j < args.n; ++j) acc += args.coef[j] * args.insc[j][s];
    outsc[s] = basesc[s] + scd * acc;
  }
}

// field_new and the two error sums of one DOPRI853 try (dopri853.c:438-486).
// k[0..7] = stages 1, 6, 7, 8, 9, 10, 11, 12.
struct FinalArgs {
  const void *k[8];
  const double *ksc[8];
  double b[8], e5[8], e3[8];  // e5 = b - bhh on stages 1, 9, 12
  const double *dt;           // step size (device memory)
  double rtol, atol;
  double noise;               // eta * eps32 (mixed form), 0 for FP64
  long long next;             // Next (tensor segment length)
  double *diag;               // per-segment sums [phi, dphi, psi, dpsi, h, dh] x (e5, e3), or null
};

// The final combination and both embedded error sums in one pass
// (dopri853.c:436-458, error() 469-486).  The FP64 homogeneous parts of the
// three combinations are formed once per CTA in shared memory; per element
// the work is FP32 (mixed form, rounding floor removed) or FP64, and the
// squared ratios are accumulated in FP64 per thread.
template <typename T, bool DIAG>
__global__ void __launch_bounds__(256) k_dopri_final(const T *__restrict__ y, const double *ysc, T *__restrict__ ynew,
                              double *ynsc, FinalArgs a, long long N, long long nf,
                              double *partials) {
  constexpr int W = Vec4<T>::W;
  const long long nv = nf / W;
  // homogeneous parts: sb, s5, s3, y, ynew of the 5 FP64 scalars
  __shared__ double hs[5][5];
  const double dt = *a.dt;
  if (threadIdx.x < 5) {
    const int sidx = threadIdx.x;
    double x = 0.0, e5 = 0.0, e3 = 0.0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const double kv = a.ksc[j][sidx];
      x += a.b[j] * kv;
      e5 += a.e5[j] * kv;
      e3 += a.e3[j] * kv;
    }
    hs[0][sidx] = x;
    hs[1][sidx] = e5;
    hs[2][sidx] = e3;
    hs[3][sidx] = ysc[sidx];
    hs[4][sidx] = ysc[sidx] + dt * x;
  }
  __syncthreads();
  T cb[8], c5[8], c3[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    cb[j] = (T)a.b[j];
    c5[j] = (T)a.e5[j];
    c3[j] = (T)a.e3[j];
  }
  const T dtT = (T)dt;
  const T atolT = (T)a.atol, rtolT = (T)a.rtol;
  const long long N2 = 2 * N, N3 = 3 * N, N4 = 4 * N, Nh = 4 * N + 2 * a.next;
  // mixed form, dh segment: the FP32 transforms of the tensor sources leave
  // absolute noise of the order of eps32 * max|dh'| on every mode, which the
  // per-element floor (relative to |c_j k_j|) misses on the small modes; the
  // error sums drop sum_j |c_j| * eta * eps32 * max|dh'_j| there as well
  // (max|dh'_j| in slot 7 of the stage's homogeneous parts)
  T nabs5 = 0, nabs3 = 0;
  if constexpr (sizeof(T) == 4) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const float mj = (float)a.ksc[j][7];
      nabs5 += fabsf(c5[j]) * mj;
      nabs3 += fabsf(c3[j]) * mj;
    }
    nabs5 *= (float)a.noise;
    nabs3 *= (float)a.noise;
  }
  double err = 0.0, err2 = 0.0;
  double dacc[DIAG ? 12 : 1];
#pragma unroll
  for (int i = 0; i < (DIAG ? 12 : 1); ++i) dacc[i] = 0.0;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv;
       v += (long long)gridDim.x * blockDim.x) {
    T ab[W], a5[W], a3[W], t5[W], t3[W], x[W];
#pragma unroll
    for (int w = 0; w < W; ++w) ab[w] = a5[w] = a3[w] = t5[w] = t3[w] = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      vload<T>((const T *)a.k[j] + v * W, x);
#pragma unroll
      for (int w = 0; w < W; ++w) {
        ab[w] += cb[j] * x[w];
        a5[w] += c5[j] * x[w];
        a3[w] += c3[j] * x[w];
        if constexpr (sizeof(T) == 4) {
          t5[w] += fabsf(c5[j] * x[w]);
          t3[w] += fabsf(c3[j] * x[w]);
        }
      }
    }
    T yv[W], yn[W];
    vload<T>(y + v * W, yv);
#pragma unroll
    for (int w = 0; w < W; ++w) yn[w] = yv[w] + dtT * ab[w];
    vstore<T>(ynew + v * W, yn);
    const long long i0 = v * W;
    // W divides N: a vector lies in one segment
    const int seg = i0 < N ? 0 : (i0 < N2 ? 1 : (i0 < N3 ? 2 : (i0 < N4 ? 3 : 4)));
    double acc5d, acc3d;
    if constexpr (sizeof(T) == 4) {
      // mixed form: per-element arithmetic in FP32, FP32 rounding floor removed
      const float nz = (float)a.noise;
      const float ys = seg < 4 ? (float)hs[3][seg] : 0.f, yns = seg < 4 ? (float)hs[4][seg] : 0.f;
      const float q5s = seg < 4 ? (float)hs[1][seg] : 0.f, q3s = seg < 4 ? (float)hs[2][seg] : 0.f;
      const bool dh = i0 >= Nh;
      const float fa5 = dh ? (float)nabs5 : 0.f, fa3 = dh ? (float)nabs3 : 0.f;
      float acc5 = 0.f, acc3 = 0.f;
#pragma unroll
      for (int w = 0; w < W; ++w) {
        const float f5 = fmaxf(fabsf(a5[w]) - nz * t5[w] - fa5, 0.f);
        const float f3 = fmaxf(fabsf(a3[w]) - nz * t3[w] - fa3, 0.f);
        const float q5 = copysignf(f5, a5[w]) + q5s, q3 = copysignf(f3, a3[w]) + q3s;
        const float isk = __frcp_rn(atolT + rtolT * fmaxf(fabsf(ys + yv[w]), fabsf(yns + yn[w])));
        const float r5 = q5 * isk, r3 = q3 * isk;
        acc5 += r5 * r5;
        acc3 += r3 * r3;
      }
      acc5d = (double)acc5;
      acc3d = (double)acc3;
    } else {
      const double ys = seg < 4 ? hs[3][seg] : 0.0, yns = seg < 4 ? hs[4][seg] : 0.0;
      const double q5s = seg < 4 ? hs[1][seg] : 0.0, q3s = seg < 4 ? hs[2][seg] : 0.0;
      acc5d = 0.0;
      acc3d = 0.0;
#pragma unroll
      for (int w = 0; w < W; ++w) {
        const double q5 = (double)a5[w] + q5s, q3 = (double)a3[w] + q3s;
        const double sk = a.atol + a.rtol * fmax(fabs((double)yv[w] + ys), fabs((double)yn[w] + yns));
        const double r5 = q5 / sk, r3 = q3 / sk;
        acc5d += r5 * r5;
        acc3d += r3 * r3;
      }
    }
    err2 += acc5d;
    err += acc3d;
    if constexpr (DIAG) {
      const int cls = seg < 4 ? seg : (i0 < Nh ? 4 : 5);
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        if (q == cls) {
          dacc[2 * q] += acc5d;
          dacc[2 * q + 1] += acc3d;
        }
      }
    }
  }
  if constexpr (DIAG) {
#pragma unroll
    for (int i = 0; i < 12; ++i)
      if (dacc[i] != 0.0) atomicAdd(&a.diag[i], dacc[i]);
  }
  double ysv[5], ynv[5], s5[5], s3[5];
#pragma unroll
  for (int q = 0; q < 5; ++q) {
    ysv[q] = hs[3][q];
    ynv[q] = hs[4][q];
    s5[q] = hs[1][q];
    s3[q] = hs[2][q];
  }
  // scale factor a (the last state component)
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const double sk = a.atol + a.rtol * fmax(fabs(ysv[4]), fabs(ynv[4]));
    const double r5 = s5[4] / sk, r3 = s3[4] / sk;
    err2 += r5 * r5;
    err += r3 * r3;
#pragma unroll
    for (int s = 0; s < 5; ++s) ynsc[s] = ynv[s];
    ynsc[5] = ynsc[6] = ynsc[7] = 0.0;
  }
  // block reduction
  for (int o = 16; o > 0; o >>= 1) {
    err += __shfl_down_sync(0xffffffffu, err, o);
    err2 += __shfl_down_sync(0xffffffffu, err2, o);
  }
  __shared__ double red[2][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][wid] = err;
    red[1][wid] = err2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0.0, s1 = 0.0;
    for (int w = 0; w < (int)(blockDim.x / 32); ++w) {
      s0 += red[0][w];
      s1 += red[1][w];
    }
    partials[2 * blockIdx.x] = s0;
    partials[2 * blockIdx.x + 1] = s1;
  }
}

// error() (dopri853.c:469-486) -> out[0]; <rho> and the NaN flag of the last
// RHS -> out[1], out[2]
__global__ void k_dopri_err_finish(const double *partials, int nb, const double *dtp, double ntot,
                                   const RhsScalars *rs, const int *waitflag, double *out) {
  const double dt = *dtp;
  double e = 0.0, e2 = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    e += partials[2 * b];
    e2 += partials[2 * b + 1];
  }
  __shared__ double sh[2][32];
  for (int o = 16; o > 0; o >>= 1) {
    e += __shfl_down_sync(0xffffffffu, e, o);
    e2 += __shfl_down_sync(0xffffffffu, e2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    sh[0][threadIdx.x >> 5] = e;
    sh[1][threadIdx.x >> 5] = e2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double err = 0.0, err2 = 0.0;
    for (int w = 0; w < (int)(blockDim.x / 32); ++w) {
      err += sh[0][w];
      err2 += sh[1][w];
    }
    double deno = err + 0.01 * err2;
    if (deno <= 0.0) deno = 1.0;
    out[0] = dt * err * sqrt(1.0 / (ntot * deno));
    out[1] = rs->rho_mean;
    // 2: a bounded device-side wait of this try timed out; 1: NaN/Inf
    out[2] = (waitflag && *waitflag) ? 2.0 : ((rs->nonfinite || !isfinite(out[0])) ? 1.0 : 0.0);
  }
}

static unsigned stream_grid(long long nvec) {
  // a multiple of the 152 SMs, at most 8 CTAs per SM
  long long b = (nvec + 255) / 256;
  long long cap = 152LL * 8;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

// ---------------------------------------------------------------------------
// Velocity form of the stage combinations (the mixed form).  Three pairs of
// state segments are (position, velocity) with position' = velocity in the
// RHS -- (phi, Pi), (psi, dpsi), (h, dh), toolbox.c:282-299, 311-346 -- so
// the position half of every stage vector is the velocity half of its stage
// input, k_j^p = Y_j^v = y^v + dt sum_l a_jl k_l^v.  Hence
//   Y_s^p  = y^p + dt (sum_j a_sj) y^v + dt^2 sum_l (A^2)_sl k_l^v,
//   ynew^p = y^p + dt (sum_j b_j) y^v + dt^2 sum_l (b^T A)_l k_l^v,
//   err^p  = (sum_j e_j) y^v + dt sum_l (e^T A)_l k_l^v   (e = e5, e3),
// the reference's combinations (dopri853.c:340-486) in exact arithmetic, with
// only the velocity halves of the stage vectors read (about 13 GB less per
// try at 256^3).  The FP64 form keeps the reference's formulation.

// position / velocity element pairs, W at a time (region boundaries are
// multiples of W): (phi, Pi), (psi, dpsi) over N, (h1, dh1), (h2, dh2) over
// Next; segment classes 0 phi, 1 Pi, 2 psi, 3 dpsi, 4 h, 5 dh
__device__ __forceinline__ void vel_pair(long long q, long long N, long long Next, long long &ip,
                                         long long &iv, int &cp, int &cv) {
  if (q < N) {
    ip = q;
    iv = N + q;
    cp = 0;
    cv = 1;
  } else if (q < 2 * N) {
    ip = N + q;
    iv = 2 * N + q;
    cp = 2;
    cv = 3;
  } else if (q < 2 * N + Next) {
    const long long e = q - 2 * N;
    ip = 4 * N + e;
    iv = 4 * N + 2 * Next + e;
    cp = 4;
    cv = 5;
  } else {
    const long long e = q - 2 * N - Next;
    ip = 4 * N + Next + e;
    iv = 4 * N + 3 * Next + e;
    cp = 4;
    cv = 5;
  }
}

struct VelLin {
  const void *k[kMaxTerms];       // stage vectors (velocity halves read)
  const double *ksc[kMaxTerms];
  double cv[kMaxTerms];           // a_sl (velocity; the homogeneous parts)
  float cvf[kMaxTerms], cpf[kMaxTerms];  // a_sl and (A^2)_sl in FP32
  float csf;                      // sum_l a_sl
  int n;
  const double *dt;
};

// position half of a velocity-form stage vector, k_j^p = Y_j^v, from the
// velocity halves its stage input was formed from (the accumulation of
// k_lincomb_vel), for the dense output, which reads whole stage vectors
__global__ void k_restore_pos(const float *__restrict__ y, float *__restrict__ kout,
                              const VelLin a, float dt, long long N, long long Next) {
  const long long nq = (2 * N + 2 * Next) / 4;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nq;
       v += (long long)gridDim.x * blockDim.x) {
    long long ip, iv;
    int c0, c1;
    vel_pair(v * 4, N, Next, ip, iv, c0, c1);
    float av[4] = {0.f, 0.f, 0.f, 0.f}, x[4];
#pragma unroll
    for (int j = 0; j < kMaxTerms; ++j) {
      if (j < a.n) {
        vload<float>((const float *)a.k[j] + iv, x);
#pragma unroll
        for (int w = 0; w < 4; ++w) av[w] += a.cvf[j] * x[w];
      }
    }
    float yv[4], ov[4];
    vload<float>(y + iv, yv);
#pragma unroll
    for (int w = 0; w < 4; ++w) ov[w] = yv[w] + dt * av[w];
    vstore<float>(kout + ip, ov);
  }
}

__global__ void k_lincomb_vel(const float *__restrict__ y, const double *ysc,
                              float *__restrict__ out, double *outsc, const VelLin a, long long N,
                              long long Next) {
  const long long nq = (2 * N + 2 * Next) / 4;
  const double dtd = *a.dt;
  const float dt = (float)dtd;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nq;
       v += (long long)gridDim.x * blockDim.x) {
    long long ip, iv;
    int c0, c1;
    vel_pair(v * 4, N, Next, ip, iv, c0, c1);
    float av[4] = {0.f, 0.f, 0.f, 0.f}, ap[4] = {0.f, 0.f, 0.f, 0.f}, x[4];
#pragma unroll
    for (int j = 0; j < kMaxTerms; ++j) {
      if (j < a.n) {
        vload<float>((const float *)a.k[j] + iv, x);
#pragma unroll
        for (int w = 0; w < 4; ++w) {
          av[w] += a.cvf[j] * x[w];
          ap[w] += a.cpf[j] * x[w];
        }
      }
    }
    float yp[4], yv[4], op[4], ov[4];
    vload<float>(y + ip, yp);
    vload<float>(y + iv, yv);
#pragma unroll
    for (int w = 0; w < 4; ++w) {
      ov[w] = yv[w] + dt * av[w];
      op[w] = yp[w] + dt * (a.csf * yv[w] + dt * ap[w]);
    }
    vstore<float>(out + iv, ov);
    vstore<float>(out + ip, op);
  }
  if (blockIdx.x == 0 && threadIdx.x < 5) {
    const int s = threadIdx.x;
    double acc = 0.0;
    for (int j = 0; j < a.n; ++j) acc += a.cv[j] * a.ksc[j][s];
    outsc[s] = ysc[s] + dtd * acc;
  }
}

constexpr int kFinalVelStages = 10;  // DOPRI853 stages 1, 4..12

struct FinalVel {
  const void *k[12];              // the stages with a nonzero coefficient
  const double *ksc[12];
  double b[12], e5[12], e3[12];   // velocity weights (and the homogeneous parts)
  float bf[12], e5f[12], e3f[12];
  float bpf[12], e5pf[12], e3pf[12];  // (b^T A)_l, (e5^T A)_l, (e3^T A)_l
  float sbf, s5f, s3f;            // sum_l b_l, e5_l, e3_l
  int n;
  const double *dt;
  double rtol, atol, noise;
  long long next;
  double *diag;
};

// NS = a.n stages (10 for DOPRI853: stages 1, 4..12), all loads of an
// element group issued before its arithmetic
template <int NS, bool DIAG>
__global__ void __launch_bounds__(256, 2) k_dopri_final_vel(const float *__restrict__ y, const double *ysc,
                                  float *__restrict__ ynew, double *ynsc, const FinalVel a,
                                  long long N, double *partials) {
  __shared__ double hs[5][5];
  const double dt = *a.dt;
  if (threadIdx.x < 5) {  // homogeneous parts: full weights on every stage's scalars
    const int sidx = threadIdx.x;
    double x = 0.0, e5 = 0.0, e3 = 0.0;
    for (int j = 0; j < a.n; ++j) {
      const double kv = a.ksc[j][sidx];
      x += a.b[j] * kv;
      e5 += a.e5[j] * kv;
      e3 += a.e3[j] * kv;
    }
    hs[0][sidx] = x;
    hs[1][sidx] = e5;
    hs[2][sidx] = e3;
    hs[3][sidx] = ysc[sidx];
    hs[4][sidx] = ysc[sidx] + dt * x;
  }
  __syncthreads();
  const float dtf = (float)dt;
  const float atolf = (float)a.atol, rtolf = (float)a.rtol, nz = (float)a.noise;
  // absolute floors from max|dh'| of each stage (slot 7): dh (velocity) and h
  float nab5v = 0.f, nab3v = 0.f, nab5p = 0.f, nab3p = 0.f;
  for (int j = 0; j < a.n; ++j) {
    const float mj = (float)a.ksc[j][7];
    nab5v += fabsf(a.e5f[j]) * mj;
    nab3v += fabsf(a.e3f[j]) * mj;
    nab5p += fabsf(a.e5pf[j]) * mj;
    nab3p += fabsf(a.e3pf[j]) * mj;
  }
  nab5v *= nz;
  nab3v *= nz;
  nab5p *= nz * dtf;
  nab3p *= nz * dtf;
  const long long Next = a.next;
  const long long nq = (2 * N + 2 * Next) / 4;
  double err = 0.0, err2 = 0.0;
  double dacc[DIAG ? 12 : 1];
#pragma unroll
  for (int i = 0; i < (DIAG ? 12 : 1); ++i) dacc[i] = 0.0;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nq;
       v += (long long)gridDim.x * blockDim.x) {
    long long ip, iv;
    int c0, c1;
    vel_pair(v * 4, N, Next, ip, iv, c0, c1);
    float4 xs[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) xs[j] = *reinterpret_cast<const float4 *>((const float *)a.k[j] + iv);
    float yp[4], yv[4], np[4], nv[4];
    vload<float>(y + ip, yp);
    vload<float>(y + iv, yv);
    float bv[4] = {}, f5v[4] = {}, f3v[4] = {}, t5v[4] = {}, t3v[4] = {};
    float bp[4] = {}, f5p[4] = {}, f3p[4] = {}, t5p[4] = {}, t3p[4] = {};
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      const float x[4] = {xs[j].x, xs[j].y, xs[j].z, xs[j].w};
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        bv[w] += a.bf[j] * x[w];
        f5v[w] += a.e5f[j] * x[w];
        f3v[w] += a.e3f[j] * x[w];
        t5v[w] += fabsf(a.e5f[j] * x[w]);
        t3v[w] += fabsf(a.e3f[j] * x[w]);
        bp[w] += a.bpf[j] * x[w];
        f5p[w] += a.e5pf[j] * x[w];
        f3p[w] += a.e3pf[j] * x[w];
        t5p[w] += fabsf(a.e5pf[j] * x[w]);
        t3p[w] += fabsf(a.e3pf[j] * x[w]);
      }
    }
#pragma unroll
    for (int w = 0; w < 4; ++w) {
      nv[w] = yv[w] + dtf * bv[w];
      np[w] = yp[w] + dtf * (a.sbf * yv[w] + dtf * bp[w]);
      // position errors: the y^v terms, then dt times the stage sums
      const float g5 = a.s5f * yv[w], g3 = a.s3f * yv[w];
      f5p[w] = g5 + dtf * f5p[w];
      f3p[w] = g3 + dtf * f3p[w];
      t5p[w] = fabsf(g5) + dtf * t5p[w];
      t3p[w] = fabsf(g3) + dtf * t3p[w];
    }
    vstore<float>(ynew + iv, nv);
    vstore<float>(ynew + ip, np);
    // the two elements of each pair: FP32 rounding floors removed, FP64 norm
    double acc5[2] = {0.0, 0.0}, acc3[2] = {0.0, 0.0};
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int cls = half ? c1 : c0;
      const int seg = cls < 4 ? cls : 4;
      const float ys = seg < 4 ? (float)hs[3][seg] : 0.f, yns = seg < 4 ? (float)hs[4][seg] : 0.f;
      const float q5s = seg < 4 ? (float)hs[1][seg] : 0.f, q3s = seg < 4 ? (float)hs[2][seg] : 0.f;
      const float fa5 = cls == 5 ? nab5v : (cls == 4 ? nab5p : 0.f);
      const float fa3 = cls == 5 ? nab3v : (cls == 4 ? nab3p : 0.f);
      float a5s = 0.f, a3s = 0.f;
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        const float e5 = half ? f5v[w] : f5p[w], e3 = half ? f3v[w] : f3p[w];
        const float s5 = half ? t5v[w] : t5p[w], s3 = half ? t3v[w] : t3p[w];
        const float yo = half ? yv[w] : yp[w], yn = half ? nv[w] : np[w];
        const float r5a = fmaxf(fabsf(e5) - nz * s5 - fa5, 0.f);
        const float r3a = fmaxf(fabsf(e3) - nz * s3 - fa3, 0.f);
        const float q5 = copysignf(r5a, e5) + q5s, q3 = copysignf(r3a, e3) + q3s;
        const float isk = __frcp_rn(atolf + rtolf * fmaxf(fabsf(ys + yo), fabsf(yns + yn)));
        const float r5 = q5 * isk, r3 = q3 * isk;
        a5s += r5 * r5;
        a3s += r3 * r3;
      }
      acc5[half] = (double)a5s;
      acc3[half] = (double)a3s;
    }
    err2 += acc5[0] + acc5[1];
    err += acc3[0] + acc3[1];
    if constexpr (DIAG) {
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        if (q == c0) {
          dacc[2 * q] += acc5[0];
          dacc[2 * q + 1] += acc3[0];
        }
        if (q == c1) {
          dacc[2 * q] += acc5[1];
          dacc[2 * q + 1] += acc3[1];
        }
      }
    }
  }
  if constexpr (DIAG) {
#pragma unroll
    for (int i = 0; i < 12; ++i)
      if (dacc[i] != 0.0) atomicAdd(&a.diag[i], dacc[i]);
  }
  // scale factor a (the last state component), the new homogeneous parts
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const double sk = a.atol + a.rtol * fmax(fabs(hs[3][4]), fabs(hs[4][4]));
    const double r5 = hs[1][4] / sk, r3 = hs[2][4] / sk;
    err2 += r5 * r5;
    err += r3 * r3;
#pragma unroll
    for (int q = 0; q < 5; ++q) ynsc[q] = hs[4][q];
    ynsc[5] = ynsc[6] = ynsc[7] = 0.0;
  }
  for (int o = 16; o > 0; o >>= 1) {
    err += __shfl_down_sync(0xffffffffu, err, o);
    err2 += __shfl_down_sync(0xffffffffu, err2, o);
  }
  __shared__ double red[2][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][wid] = err;
    red[1][wid] = err2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double e = 0.0, e2 = 0.0;
    for (int w = 0; w < (int)(blockDim.x / 32); ++w) {
      e += red[0][w];
      e2 += red[1][w];
    }
    partials[2 * blockIdx.x] = e;
    partials[2 * blockIdx.x + 1] = e2;
  }
}

static int lincomb(Ctx *c, const Vec &base, Vec &out, const LinArgs &args) {
  const long long nf = c->g.Nf;
  prof_begin(c, KK_LINCOMB);
  if (c->mixed) {
    k_lincomb<float><<<stream_grid(nf / 4), 256, 0, c->stream>>>(
        (const float *)base.fl, base.sc, (float *)out.fl, out.sc, args, nf);
  } else {
    k_lincomb<double><<<stream_grid(nf / 2), 256, 0, c->stream>>>(
        (const double *)base.fl, base.sc, (double *)out.fl, out.sc, args, nf);
  }
  prof_end(c, KK_LINCOMB, (double)(args.n + 2) * nf * c->tsize);
  return check_launch(c, "k_lincomb");
}

static int alloc_vec(Ctx *c, Vec &v) {
  if (v.fl) return IH_OK;
  IH_CUDA(c, cudaMalloc(&v.fl, c->tsize * c->g.Nf));
  IH_CUDA(c, cudaMemsetAsync(v.fl, 0, c->tsize * c->g.Nf, c->stream));
  IH_CUDA(c, cudaMalloc((void **)&v.sc, sizeof(double) * kSc));
  IH_CUDA(c, cudaMemsetAsync(v.sc, 0, sizeof(double) * kSc, c->stream));
  c->dev_bytes += c->tsize * c->g.Nf + sizeof(double) * kSc;
  return IH_OK;
}

// Features of the last accepted step: log dt_n..dt_{n-3}, log err_n..err_{n-3},
// log a, H, log rms(delta phi), log rms(delta psi).  Missing history entries
// repeat the oldest available one.
int step_features(Ctx *c, float *out) {
  if (c->hist_n < 1) {
    c->err = "no accepted step yet";
    return IH_ERR_STATE;
  }
  double *d = c->diag + 4 * c->g.bins + 100;  // 2 doubles: rms phi, rms psi
  IH_TRY(field_rms(c, c->y.fl, c->g.N, d));
  IH_TRY(field_rms(c, (const char *)c->y.fl + 2 * c->g.N * c->tsize, c->g.N, d + 1));
  IH_CUDA(c, cudaMemcpyAsync(c->hpin, d, sizeof(double) * 2, cudaMemcpyDeviceToHost, c->stream));
  IH_CUDA(c, cudaMemcpyAsync(c->hpin + 2, c->y.sc + 4, sizeof(double), cudaMemcpyDeviceToHost,
                             c->stream));
  IH_CUDA(c, cudaMemcpyAsync(c->hpin + 3, (const char *)c->rs + offsetof(RhsScalars, H),
                             sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  const int n = c->hist_n < 4 ? c->hist_n : 4;
  for (int i = 0; i < 4; ++i) {
    const int k = i < n ? i : n - 1;
    out[i] = (float)log(c->hist_dt[k]);
    out[4 + i] = (float)log(fmax(c->hist_err[k], 1e-10));
  }
  out[8] = (float)log(c->hpin[2]);
  out[9] = (float)c->hpin[3];
  out[10] = (float)log(fmax(c->hpin[0], 1e-300));
  out[11] = (float)log(fmax(c->hpin[1], 1e-300));
  return IH_OK;
}

// the reference controller's next step after an accepted try of error err
// (success(), dopri853.c:505-530): the scale safe err^-alpha err_old^beta in
// [minscale, maxscale], not above 1 right after a rejection, then the Hubble
// cap
static double controller_next(const ih_dopri_cfg &g, double err, double err_old,
                              bool after_reject, double dt, double rho_mean) {
  const double alpha = 1.0 / 8.0 - g.beta * 0.2;
  double scale;
  if (err == 0.0) {
    scale = g.maxscale;
  } else {
    scale = g.safe * pow(err, -alpha) * pow(err_old, g.beta);
    if (scale < g.minscale) scale = g.minscale;
    if (scale > g.maxscale) scale = g.maxscale;
  }
  double next = after_reject ? dt * fmin(scale, 1.0) : dt * scale;
  if (g.max_dt_hubble_fraction > 0.0) {
    const double minstep = g.max_dt_hubble_fraction * sqrt(3.0 / rho_mean);
    if (next > minstep) next = minstep;
  }
  return next;
}

// the learned proposal for the next step (after an accepted step): the
// network's log dt, clamped to [minscale, maxscale] x the step just taken and
// to the Hubble cap
static int learned_dt(Ctx *c, double dt_did, double rho_mean, double *dt_out) {
  float f[IH_MLP_INPUTS];
  IH_TRY(step_features(c, f));
  IH_CUDA(c, cudaMemcpyAsync(c->feat_dev, f, sizeof f, cudaMemcpyHostToDevice, c->stream));
  IH_TRY(mlp_forward_async(c->proposer, c->feat_dev, 1, c->feat_dev + 12, c->stream));
  float ylog = 0.f;
  IH_CUDA(c, cudaMemcpyAsync(&ylog, c->feat_dev + 12, sizeof(float), cudaMemcpyDeviceToHost,
                             c->stream));
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  double dt = exp((double)ylog);
  if (!(dt > 0.0) || !isfinite(dt)) dt = c->dt_next_pi;  // fall back to the controller
  dt = fmin(fmax(dt, dt_did * c->cfg.minscale), dt_did * c->cfg.maxscale);
  if (c->cfg.max_dt_hubble_fraction > 0.0)
    dt = fmin(dt, c->cfg.max_dt_hubble_fraction * sqrt(3.0 / rho_mean));
  *dt_out = dt;
  return IH_OK;
}

int dopri_init(Ctx *c, const ih_dopri_cfg *cfg, double t0, double dt0, int want_output) {
  tableau_init();
  for (int j = 1; j <= 12; ++j) IH_TRY(alloc_vec(c, c->k[j]));
  c->cfg = *cfg;
  c->t = t0;
  c->dt_next = dt0;
  c->err_old = 1.0e-4;
  c->reject = 0;
  c->n_ok = c->n_bad = c->n_stp = c->n_tries = 0;
  c->hist_n = 0;
  c->dense_ready = 0;
  // prepare_and_save_timeslice: RHS with the filter on (toolbox.c:96-104)
  IH_TRY(rhs(c, t0, c->y, c->k[1], 1, want_output, nullptr));
  c->dopri_ready = 1;
  return IH_OK;
}

// try_step + error (dopri853.c:331-486); returns err via *err_out
// One DOPRI853 try on the device (dopri853.c:331-458): the 11 stage
// combinations and RHS evaluations, the final combination and the two error
// sums, reduced into diag[48..50] (error(), <rho>, the NaN flag).  The step
// size is read from c->dt_dev, so one capture serves every try.
// Tableau products of the velocity form (FP64, once): row s of try_body
// (stage s+1 from stages 1..s): VCS[s] = sum_j a_sj, VAA[s][l] =
// sum_{j=l+1}^{s-1} a_sj a_jl; final weights per stage i (0-based) and their
// products with the tableau, VBA[l] = sum_{j>l} b_j a_jl (and e5, e3).
static double VAA[12][12], VCS[12], VB[12], VE5[12], VE3[12], VBA[12], VE5A[12], VE3A[12];
static double VSB, VS5, VS3;
static std::once_flag vel_once;
static void vel_tables() {
  std::call_once(vel_once, [] {
    tableau_init();
    memset(VAA, 0, sizeof VAA);
    for (int s = 1; s < 12; ++s) {
      double cs = 0.0;
      for (int j = 0; j < s; ++j) cs += DA[s][j];
      VCS[s] = cs;
      for (int l = 0; l + 1 < s; ++l) {
        double q = 0.0;
        for (int j = l + 1; j < s; ++j) q += DA[s][j] * DA[j][l];
        VAA[s][l] = q;
      }
    }
    VSB = VS5 = VS3 = 0.0;
    for (int i = 0; i < 12; ++i) {
      const double bhh = i == 0 ? DBHH[0] : (i == 8 ? DBHH[1] : (i == 11 ? DBHH[2] : 0.0));
      VB[i] = DB[i];
      VE5[i] = DB[i] - bhh;
      VE3[i] = DE3[i];
      VSB += VB[i];
      VS5 += VE5[i];
      VS3 += VE3[i];
    }
    for (int l = 0; l < 12; ++l) {
      double b = 0.0, e5 = 0.0, e3 = 0.0;
      for (int j = l + 1; j < 12; ++j) {
        b += VB[j] * DA[j][l];
        e5 += VE5[j] * DA[j][l];
        e3 += VE3[j] * DA[j][l];
      }
      VBA[l] = b;
      VE5A[l] = e5;
      VE3A[l] = e3;
    }
  });
}

// the terms of the velocity-form input of stage s+1; stage[l] = stage l+1's
// vector (null: not available, an error if the stage has a term)
static int vel_terms(int s, const Vec *const stage[12], VelLin &a) {
  vel_tables();
  memset(&a, 0, sizeof a);
  int n = 0;
  for (int l = 0; l < s; ++l) {
    if (DA[s][l] == 0.0 && VAA[s][l] == 0.0) continue;
    if (!stage[l]) return IH_ERR_STATE;
    a.k[n] = stage[l]->fl;
    a.ksc[n] = stage[l]->sc;
    a.cv[n] = DA[s][l];
    a.cvf[n] = (float)DA[s][l];
    a.cpf[n] = (float)VAA[s][l];
    ++n;
  }
  a.n = n;
  a.csf = (float)VCS[s];
  return IH_OK;
}

// the input of stage s+1 in the velocity form (mixed form)
static int lincomb_vel(Ctx *c, int s) {
  VelLin a;
  const Vec *stage[12];
  for (int l = 0; l < 12; ++l) stage[l] = &c->k[l + 1];
  vel_terms(s, stage, a);  // every stage vector is present
  const int n = a.n;
  a.dt = c->dt_dev;
  const Geom &g = c->g;
  const long long nq = (2 * g.N + 2 * g.Next) / 4;
  prof_begin(c, KK_LINCOMB);
  k_lincomb_vel<<<stream_grid(nq), 256, 0, c->stream>>>((const float *)c->y.fl, c->y.sc,
                                                        (float *)c->ytmp.fl, c->ytmp.sc, a, g.N,
                                                        g.Next);
  prof_end(c, KK_LINCOMB, (double)(n + 4) * (g.Nf / 2) * sizeof(float));
  return check_launch(c, "k_lincomb_vel");
}

// field_new and both error sums in the velocity form (mixed form)
static int final_vel(Ctx *c) {
  vel_tables();
  FinalVel f;
  memset(&f, 0, sizeof f);
  int n = 0;
  for (int i = 0; i < 12; ++i) {
    if (VB[i] == 0.0 && VE5[i] == 0.0 && VE3[i] == 0.0 && VBA[i] == 0.0 && VE5A[i] == 0.0 &&
        VE3A[i] == 0.0)
      continue;
    f.k[n] = c->k[i + 1].fl;
    f.ksc[n] = c->k[i + 1].sc;
    f.b[n] = VB[i];
    f.e5[n] = VE5[i];
    f.e3[n] = VE3[i];
    f.bf[n] = (float)VB[i];
    f.e5f[n] = (float)VE5[i];
    f.e3f[n] = (float)VE3[i];
    f.bpf[n] = (float)VBA[i];
    f.e5pf[n] = (float)VE5A[i];
    f.e3pf[n] = (float)VE3A[i];
    ++n;
  }
  if (n != kFinalVelStages) {  // fixed by the tableau
    c->err = "velocity form: unexpected stage count of the final combination";
    return IH_ERR_STATE;
  }
  f.n = n;
  f.sbf = (float)VSB;
  f.s5f = (float)VS5;
  f.s3f = (float)VS3;
  f.dt = c->dt_dev;
  f.rtol = c->cfg.rtol;
  f.atol = c->cfg.atol;
  f.noise = c->noise_eta * 5.9604644775390625e-8;  // eta * 2^-24
  f.next = c->g.Next;
  f.diag = nullptr;
  if (c->err_diag) {
    f.diag = c->diag + 4 * c->g.bins + 64 + 8;  // 12 doubles
    IH_CUDA(c, cudaMemsetAsync(f.diag, 0, sizeof(double) * 12, c->stream));
  }
  const Geom &g = c->g;
  const long long nq = (2 * g.N + 2 * g.Next) / 4;
  const unsigned nb = stream_grid(nq);
  prof_begin(c, KK_DOPRI_FINAL);
  auto kf = f.diag ? k_dopri_final_vel<kFinalVelStages, true>
                    : k_dopri_final_vel<kFinalVelStages, false>;
  kf<<<nb, 256, 0, c->stream>>>((const float *)c->y.fl, c->y.sc, (float *)c->ynew.fl, c->ynew.sc,
                                f, g.N, c->partials);
  prof_end(c, KK_DOPRI_FINAL, (double)(n + 4) * (g.Nf / 2) * sizeof(float));
  IH_TRY(check_launch(c, "k_dopri_final_vel"));
  k_dopri_err_finish<<<1, 256, 0, c->stream>>>(c->partials, (int)nb, c->dt_dev, (double)g.Ntot,
                                               c->rs, c->waitflag, c->diag + 4 * g.bins + 48);
  return check_launch(c, "k_dopri_err_finish");
}

// The combination forming the input of iteration s of try_body (stage s+1)
// from stages 1..s, without the term of stage s when `self` is given: that
// term then comes from the RHS that writes stage s (NextLin).
static void stage_terms(Ctx *c, int s, bool self, LinArgs *a, NextLin *nl) {
  int n = 0;
  for (int j = 0; j < (self ? s - 1 : s); ++j) {
    if (DA[s][j] == 0.0) continue;
    if (a) {
      a->in[n] = c->k[j + 1].fl;
      a->insc[n] = c->k[j + 1].sc;
      a->coef[n] = DA[s][j];
    }
    if (nl) {
      nl->k[n] = c->k[j + 1].fl;
      nl->ksc[n] = c->k[j + 1].sc;
      nl->coef[n] = DA[s][j];
      nl->coeff[n] = (float)DA[s][j];
    }
    ++n;
  }
  if (a) {
    a->n = n;
    a->scale_dev = c->dt_dev;
  }
  if (nl) {
    nl->n = n;
    nl->self = DA[s][s - 1];
    nl->selff = (float)DA[s][s - 1];
    nl->base = c->y.fl;
    nl->basesc = c->y.sc;
    nl->dt = c->dt_dev;
  }
}

static int try_body(Ctx *c) {
  // With stage fusion the RHS of stage s also forms the input of stage s+1
  // (in ytmp, which it reads point by point before overwriting): one read
  // of the stage vector and one launch fewer per stage.
  // (not with the fused tensor x pass, whose variants with and without the
  // combination do not round identically)
  // (the mixed form combines stages in the velocity form instead)
  const bool vel = c->mixed && c->velocity_form;
  const bool fuse = c->stage_fusion && !c->tensor_fused && !vel;
  c->try_vel = vel ? 1 : 0;
  {
  // the velocity form reads no position half of k_2..k_12: their RHS
  // evaluations skip those copies (k_1, the FSAL vector, keeps them)
  struct SkipPos {
    Ctx *c;
    ~SkipPos() { c->skip_pos = 0; }
  } guard{c};
  c->skip_pos = vel ? 1 : 0;
  for (int s = 1; s < 12; ++s) {  // stage s+1 from stages 1..s
    if (vel) {
      IH_TRY(lincomb_vel(c, s));
    } else if (s == 1 || !fuse) {  // else the previous stage's RHS formed it
      LinArgs a;
      memset(&a, 0, sizeof a);
      stage_terms(c, s, false, &a, nullptr);
      IH_TRY(lincomb(c, c->y, c->ytmp, a));
    }
    NextLin nl;
    memset(&nl, 0, sizeof nl);
    const bool fuse_next = fuse && s + 1 < 12;
    if (fuse_next) stage_terms(c, s + 1, true, nullptr, &nl);
    // the RHS does not depend on t explicitly (toolbox.c:75-88)
    IH_TRY(rhs(c, 0.0, c->ytmp, c->k[s + 1], 0, 0, nullptr, fuse_next ? &nl : nullptr));
  }
  }
  if (vel) return final_vel(c);
  FinalArgs f;
  memset(&f, 0, sizeof f);
  const int st[8] = {1, 6, 7, 8, 9, 10, 11, 12};
  for (int j = 0; j < 8; ++j) {
    const int sidx = st[j] - 1;
    f.k[j] = c->k[st[j]].fl;
    f.ksc[j] = c->k[st[j]].sc;
    f.b[j] = DB[sidx];
    double bhh = (st[j] == 1) ? DBHH[0] : (st[j] == 9) ? DBHH[1] : (st[j] == 12) ? DBHH[2] : 0.0;
    f.e5[j] = DB[sidx] - bhh;
    f.e3[j] = DE3[sidx];
  }
  f.dt = c->dt_dev;
  f.rtol = c->cfg.rtol;
  f.atol = c->cfg.atol;
  f.noise = c->mixed ? c->noise_eta * 5.9604644775390625e-8 : 0.0;  // eta * 2^-24
  f.next = c->g.Next;
  f.diag = nullptr;
  if (c->err_diag) {
    f.diag = c->diag + 4 * c->g.bins + 64 + 8;  // 12 doubles
    IH_CUDA(c, cudaMemsetAsync(f.diag, 0, sizeof(double) * 12, c->stream));
  }
  const long long nf = c->g.Nf;
  const int W = c->mixed ? 4 : 2;
  const unsigned nb = stream_grid(nf / W);
  prof_begin(c, KK_DOPRI_FINAL);
  if (c->mixed) {
    auto kf = f.diag ? k_dopri_final<float, true> : k_dopri_final<float, false>;
    kf<<<nb, 256, 0, c->stream>>>((const float *)c->y.fl, c->y.sc, (float *)c->ynew.fl, c->ynew.sc,
                                  f, c->g.N, nf, c->partials);
  } else {
    auto kd = f.diag ? k_dopri_final<double, true> : k_dopri_final<double, false>;
    kd<<<nb, 256, 0, c->stream>>>((const double *)c->y.fl, c->y.sc, (double *)c->ynew.fl,
                                  c->ynew.sc, f, c->g.N, nf, c->partials);
  }
  prof_end(c, KK_DOPRI_FINAL, 10.0 * nf * c->tsize);
  IH_TRY(check_launch(c, "k_dopri_final"));
  k_dopri_err_finish<<<1, 256, 0, c->stream>>>(c->partials, (int)nb, c->dt_dev, (double)c->g.Ntot,
                                               c->rs, c->waitflag, c->diag + 4 * c->g.bins + 48);
  return check_launch(c, "k_dopri_err_finish");
}

// Work that is replayed as one CUDA graph per combination of the vectors it
// touches (y, ynew and the first two stage vectors swap roles after every
// accepted step).  Graphs are not used while per-kernel timing or the error
// breakdown is on; any change of what a capture bakes in (tolerances, noise
// floor, FFT engines) advances c->graph_epoch.
static bool graphs_usable(const Ctx *c) { return c->graphs_on && !c->prof_on && !c->err_diag; }

template <typename Body>
static int replay(Ctx *c, int kind, const void *const key[4], Body body) {
  Ctx::Graph *hit = nullptr;
  for (auto &gr : c->graphs)
    if (gr.kind == kind && gr.epoch == c->graph_epoch && gr.key[0] == key[0] &&
        gr.key[1] == key[1] && gr.key[2] == key[2] && gr.key[3] == key[3])
      hit = &gr;
  if (!hit) {
    const unsigned long long l0 = c->launches, r0 = c->calls_rhs;
    IH_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
    const int st = body();
    cudaGraph_t g = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(c->stream, &g);
    const unsigned long long nk = c->launches - l0, nr = c->calls_rhs - r0;
    c->launches = l0;
    c->calls_rhs = r0;
    if (st != IH_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (ee != cudaSuccess) {
      c->err = std::string("graph capture: ") + cudaGetErrorString(ee);
      return IH_ERR_CUDA;
    }
    Ctx::Graph gr;
    gr.kind = kind;
    gr.epoch = c->graph_epoch;
    for (int i = 0; i < 4; ++i) gr.key[i] = key[i];
    gr.kernels = nk;
    gr.rhs_calls = nr;
    const cudaError_t ie = cudaGraphInstantiate(&gr.exec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      c->err = std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie);
      return IH_ERR_CUDA;
    }
    c->graphs.push_back(gr);
    hit = &c->graphs.back();
  }
  IH_CUDA(c, cudaGraphLaunch(hit->exec, c->stream));
  c->launches += hit->kernels;
  c->calls_rhs += hit->rhs_calls;
  return IH_OK;
}

// try_step + error (dopri853.c:331-486) in two halves: try_enqueue queues
// the try and the read-back of its error on the context stream and returns;
// try_collect waits for them.
int try_enqueue(Ctx *c, double dt) {
  c->dense_ready = 0;  // the try overwrites the stage vectors and ynew
  c->hpin[kDtSlot] = dt;
  IH_CUDA(c, cudaMemcpyAsync(c->dt_dev, c->hpin + kDtSlot, sizeof(double), cudaMemcpyHostToDevice,
                             c->stream));
  if (graphs_usable(c)) {
    const void *key[4] = {c->y.fl, c->ynew.fl, c->k[1].fl, c->ytmp.fl};
    IH_TRY(replay(c, 0, key, [c]() { return try_body(c); }));
  } else {
    IH_TRY(try_body(c));
  }
  IH_CUDA(c, cudaMemcpyAsync(c->hpin, c->diag + 4 * c->g.bins + 48, sizeof(double) * 3,
                             cudaMemcpyDeviceToHost, c->stream));
  return IH_OK;
}

int try_collect(Ctx *c, double *err_out, double *rho_mean_out, int *nonfinite) {
  IH_CUDA(c, cudaStreamSynchronize(c->stream));
  *err_out = c->hpin[0];
  *rho_mean_out = c->hpin[1];
  *nonfinite = c->hpin[2] == 2.0 ? 2 : (c->hpin[2] != 0.0);
  return IH_OK;
}

static int try_step(Ctx *c, double dt, double *err_out, double *rho_mean_out, int *nonfinite) {
  IH_TRY(try_enqueue(c, dt));
  return try_collect(c, err_out, rho_mean_out, nonfinite);
}

// the filtered post-step RHS (dopri853.c:285-293), replayed as a graph when
// it computes no diagnostics
static int post_step_rhs(Ctx *c, double t, int want_output) {
  if (want_output || !graphs_usable(c)) return rhs(c, t, c->ynew, c->k[2], 1, want_output, &c->y);
  const void *key[4] = {c->ynew.fl, c->k[2].fl, nullptr, nullptr};
  return replay(c, 1, key, [c]() { return rhs(c, 0.0, c->ynew, c->k[2], 1, 0, &c->y); });
}

// success() (dopri853.c:505-540)
static int success(Ctx *c, double err, double rho_mean, double *dt) {
  const ih_dopri_cfg &g = c->cfg;
  const double alpha = 1.0 / 8.0 - g.beta * 0.2;
  if (err <= 1.0) {
    c->dt_next = controller_next(g, err, c->err_old, c->reject != 0, *dt, rho_mean);
    c->err_old = fmax(err, 1.0e-4);
    c->reject = 0;
    return 1;
  }
  const double scale = fmax(g.safe * pow(err, -alpha), g.minscale);
  (*dt) *= scale;
  c->reject = 1;
  return 0;
}

// The rest of perform_step once a try is accepted (dopri853.c:285-311): the
// filtered post-step RHS (queued), the swap of field/field_new and of the
// stage-1 vectors, the step history and, with a proposer, its dt_next.
int step_accept(Ctx *c, double dt, double err, double rho_mean, int want_output, int tries,
                ih_step_info *info) {
  IH_TRY(post_step_rhs(c, c->t + dt, want_output));
  Vec tmp = c->y;
  c->y = c->ynew;
  c->ynew = tmp;
  tmp = c->k[1];
  c->k[1] = c->k[2];
  c->k[2] = tmp;
  c->dense_t0 = c->t;
  c->dense_h = dt;
  c->dense_ready = 1;
  c->dense_stages = 0;
  c->dense_vel = c->try_vel;
  c->t += dt;
  c->step_start_valid = 1;
  // step history; with a proposer its proposal replaces the controller's
  for (int i = 3; i > 0; --i) {
    c->hist_dt[i] = c->hist_dt[i - 1];
    c->hist_err[i] = c->hist_err[i - 1];
  }
  c->hist_dt[0] = dt;
  c->hist_err[0] = err;
  if (c->hist_n < 4) ++c->hist_n;
  c->dt_next_pi = c->dt_next;
  if (c->proposer) IH_TRY(learned_dt(c, dt, rho_mean, &c->dt_next));
  if (info) {
    info->t = c->t;
    info->dt_did = dt;
    info->dt_next = c->dt_next;
    info->err = err;
    info->tries = tries;
    info->status = IH_OK;
  }
  return IH_OK;
}

// bookkeeping of one finished try; returns 1 when accepted (dt is then the
// accepted size), 0 to retry with the reduced dt, or an error status < 0
int try_outcome(Ctx *c, double err, double rho_mean, int nonfinite, double *dt) {
  ++c->n_tries;
  c->last_err = err;
  if (nonfinite == 2) {
    c->err = "a device-side wait timed out (TMA load of a tensor-source plane); results void";
    return -IH_ERR_CUDA;
  }
  if (nonfinite) {
    c->err = "non-finite value in the RHS reductions or the error norm";
    return -IH_ERR_NAN;
  }
  if (success(c, err, rho_mean, dt)) return 1;
  if (fabs(*dt) <= fabs(c->t) * DBL_EPSILON) {
    c->err = "step size underflow";
    return -IH_ERR_UNDERFLOW;
  }
  return 0;
}

int dopri_step(Ctx *c, double dt_try, int want_output, ih_step_info *info) {
  if (!c->dopri_ready) {
    c->err = "ih_dopri853_init has not been called";
    return IH_ERR_STATE;
  }
  double dt = dt_try;
  int tries = 0;
  double err = 0.0, rho_mean = 0.0;
  for (;;) {
    int nonfinite;
    IH_TRY(try_step(c, dt, &err, &rho_mean, &nonfinite));
    ++tries;
    const int o = try_outcome(c, err, rho_mean, nonfinite, &dt);
    if (o == 1) break;
    if (o < 0) {
      if (info) {
        info->status = -o;
        info->tries = tries;
      }
      return -o;
    }
  }
  return step_accept(c, dt, err, rho_mean, want_output, tries, info);
}

// The DOP853 continuous extension of the last accepted step at t_out in
// [t - dt_did, t] (Hairer, Norsett & Wanner; coefficients
// dopri853_constants.c:23-25, 98-173).  Ingredients after step_accept: the
// step's start state in ynew, field_new (after the post-step RHS, filtered
// in place when the filter is on) in y, stage 1 in k[2], stages 3..12 in
// k[3..12], stage 13 = f(field_new) in k[1]; stages 14..16 are evaluated
// once per step into kd[0..2].  The interpolant
//   r1 + th (r2 + s (r3 + th (r4 + s (r5 + th (r6 + s (r7 + th r8)))))),
//   s = 1 - th, r1 = y0, r2 = field_new - y0, r3 = h k1 - r2,
//   r4 = r2 - h k13 - r3, r(5+i) = h sum_j d(4+i)j k_j,
// is formed as y0 + h sum_j W_j k_j + u (field_new - y0) with u = th^2 (3 - 2
// th) and W_j = th^2 s^2 d4j + th^3 s^2 d5j + th^3 s^3 d6j + th^4 s^3 d7j
// (+ th s^2 on k1, - th^2 s on k13).  A velocity-form step has no position
// halves in stages 6..12; they are restored from the velocity halves first.
int dopri_dense(Ctx *c, double t_out, int want_output) {
  if (!c->dense_ready) {
    c->err = "dense output: no accepted DOPRI853 step since the last state change";
    return IH_ERR_STATE;
  }
  const double h = c->dense_h, t0 = c->dense_t0;
  double th = (t_out - t0) / h;
  const double tol = 1e-12;
  if (!(th >= -tol && th <= 1.0 + tol)) {
    c->err = "dense output: t_out outside the last accepted step";
    return IH_ERR_ARG;
  }
  th = th < 0.0 ? 0.0 : (th > 1.0 ? 1.0 : th);
  tableau_init();
  for (int r = 0; r < 3; ++r) IH_TRY(alloc_vec(c, c->kd[r]));
  IH_TRY(alloc_vec(c, c->dense));
  const Vec *st[16] = {&c->k[2], nullptr,   &c->k[3],  &c->k[4],  &c->k[5],  &c->k[6],
                       &c->k[7], &c->k[8],  &c->k[9],  &c->k[10], &c->k[11], &c->k[12],
                       &c->k[1], &c->kd[0], &c->kd[1], &c->kd[2]};
  const Vec &y0 = c->ynew;
  const Geom &g = c->g;
  if (!c->dense_stages) {
    if (c->dense_vel) {  // position halves of stages 6..12
      const Vec *vst[12];
      for (int l = 0; l < 12; ++l) vst[l] = st[l];
      for (int s = 5; s < 12; ++s) {
        VelLin a;
        if (vel_terms(s, vst, a) != IH_OK) {
          c->err = "dense output: a stage input needs stage 2, which the step no longer holds";
          return IH_ERR_STATE;
        }
        const long long nq = (2 * g.N + 2 * g.Next) / 4;
        prof_begin(c, KK_LINCOMB);
        k_restore_pos<<<stream_grid(nq), 256, 0, c->stream>>>(
            (const float *)y0.fl, (float *)c->k[s + 1].fl, a, (float)h, g.N, g.Next);
        prof_end(c, KK_LINCOMB, (double)(a.n + 2) * (g.Nf / 2) * sizeof(float));
        IH_TRY(check_launch(c, "k_restore_pos"));
      }
    }
    for (int r = 0; r < 3; ++r) {  // stages 14..16
      LinArgs a;
      memset(&a, 0, sizeof a);
      for (int j = 0; j < 13 + r; ++j) {
        if (DAD[r][j] == 0.0) continue;
        if (!st[j] || a.n == kMaxTerms) {  // fixed by the tableau: never taken
          c->err = "dense output: unexpected term list of an extra stage";
          return IH_ERR_STATE;
        }
        a.in[a.n] = st[j]->fl;
        a.insc[a.n] = st[j]->sc;
        a.coef[a.n] = DAD[r][j];
        ++a.n;
      }
      a.scale = h;
      IH_TRY(lincomb(c, y0, c->ytmp, a));
      IH_TRY(rhs(c, 0.0, c->ytmp, c->kd[r], 0, 0, nullptr, nullptr));
    }
    c->dense_stages = 1;
  }
  const double s1 = 1.0 - th;
  const double gq[4] = {th * th * s1 * s1, th * th * th * s1 * s1, th * th * th * s1 * s1 * s1,
                        th * th * th * th * s1 * s1 * s1};
  LinArgs a;
  memset(&a, 0, sizeof a);
  for (int j = 0; j < 16; ++j) {
    if (!st[j]) continue;
    double w = 0.0;
    for (int i = 0; i < 4; ++i) w += gq[i] * DDN[i][j];
    if (j == 0) w += th * s1 * s1;
    if (j == 12) w -= th * th * s1;
    if (w == 0.0) continue;
    if (a.n == kMaxTerms) {  // 12 weighted stages at most: never taken
      c->err = "dense output: unexpected term list of the interpolant";
      return IH_ERR_STATE;
    }
    a.in[a.n] = st[j]->fl;
    a.insc[a.n] = st[j]->sc;
    a.coef[a.n] = w;
    ++a.n;
  }
  a.scale = h;
  IH_TRY(lincomb(c, y0, c->ytmp, a));
  const double u = th * th * (3.0 - 2.0 * th);
  LinArgs b;
  memset(&b, 0, sizeof b);
  b.in[0] = c->y.fl;
  b.insc[0] = c->y.sc;
  b.coef[0] = u;
  b.in[1] = y0.fl;
  b.insc[1] = y0.sc;
  b.coef[1] = -u;
  b.n = 2;
  b.scale = 1.0;
  IH_TRY(lincomb(c, c->ytmp, c->dense, b));
  // the output RHS of a saved slice (filtered, diagnostics kept), on the copy
  if (want_output) IH_TRY(rhs(c, t_out, c->dense, c->ytmp, 1, 1, nullptr));
  return IH_OK;
}

// rk4.c:108-161 (one step)
int rk4_step(Ctx *c, double dt, int want_output) {
  c->dense_ready = 0;
  for (int j = 1; j <= 4; ++j) IH_TRY(alloc_vec(c, c->k[j]));
  const double t = c->t;
  IH_TRY(rhs(c, t, c->y, c->k[1], 1, want_output, nullptr));
  LinArgs a;
  memset(&a, 0, sizeof a);
  a.n = 1;
  a.coef[0] = 0.5;
  a.in[0] = c->k[1].fl;
  a.insc[0] = c->k[1].sc;
  a.scale = dt;
  IH_TRY(lincomb(c, c->y, c->ytmp, a));
  IH_TRY(rhs(c, t + dt / 2.0, c->ytmp, c->k[2], 0, 0, nullptr));
  a.in[0] = c->k[2].fl;
  a.insc[0] = c->k[2].sc;
  IH_TRY(lincomb(c, c->y, c->ytmp, a));
  IH_TRY(rhs(c, t + dt / 2.0, c->ytmp, c->k[3], 0, 0, nullptr));
  a.in[0] = c->k[3].fl;
  a.insc[0] = c->k[3].sc;
  a.coef[0] = 1.0;
  IH_TRY(lincomb(c, c->y, c->ytmp, a));
  IH_TRY(rhs(c, t + dt, c->ytmp, c->k[4], 0, 0, nullptr));
  LinArgs f;
  memset(&f, 0, sizeof f);
  f.n = 4;
  const double w[4] = {1.0 / 6.0, 2.0 / 6.0, 2.0 / 6.0, 1.0 / 6.0};
  for (int j = 0; j < 4; ++j) {
    f.in[j] = c->k[j + 1].fl;
    f.insc[j] = c->k[j + 1].sc;
    f.coef[j] = w[j];
  }
  f.scale = dt;
  IH_TRY(lincomb(c, c->y, c->ynew, f));
  Vec tmp = c->y;
  c->y = c->ynew;
  c->ynew = tmp;
  c->t = t + dt;
  c->step_start_valid = 1;
  return IH_OK;
}

}  // namespace ih
