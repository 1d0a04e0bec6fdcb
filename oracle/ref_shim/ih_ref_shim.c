/*
 * ih_ref_shim.c -- implementations behind the shim headers fftw3.h, hdf5.h
 * and the gsl/ headers, so that nikikilbertus/InstaHeat's own src/ C files compile and run
 * unmodified as the second oracle (oracle/_ref, built by oracle/ref.py).
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links this file.
 *
 *  - FFTW3 subset over the oracle's FP64 Stockham transforms
 *    (ih_oracle_fft.c); the reference's plans are 1-, 2- or 3-dimensional
 *    (setup.c:524-554) and all map onto the oracle's [nx][ny][nz] real
 *    transform with leading extents of 1.
 *  - HDF5 recorder: datasets live in memory (rank <= 2 hyperslab writes and
 *    reads, as io.c uses them); H5Fclose / H5Fflush write them to the path
 *    given to H5Fcreate in the record format
 *        "IHH5REC1", then per dataset: u32 name length, name, u32 class
 *        (0 double, 1 string), u32 rank, u64 dims[rank], u64 byte count,
 *        the bytes (doubles in native byte order),
 *    and H5Fopen reads that format back.
 *  - GSL: MT19937 (Matsumoto and Nishimura 1998, initialisation of 2002) as
 *    GSL documents gsl_rng_set / gsl_rng_uniform; the quadrature and spline
 *    calls of the Bunch-Davies path report GSL_EUNIMPL.
 */
#include <complex.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3.h"
#include "hdf5.h"
#include "gsl/gsl_errno.h"
#include "gsl/gsl_integration.h"
#include "gsl/gsl_rng.h"
#include "gsl/gsl_spline.h"
#include "../ih_oracle_internal.h"

static void shim_fail(const char *what)
{
    fprintf(stderr, "reference shim: %s\n", what);
    exit(EXIT_FAILURE);
}

/* ------------------------------------------------------------------ FFTW */

struct ih_ref_fftw_plan_s {
    int dir;          /* FFTW_FORWARD: r2c, FFTW_BACKWARD: c2r */
    size_t nreal;     /* real points */
    size_t ncomplex;  /* half-spectrum points */
    iho_fft3 F;
    double *real_arr; /* arrays given at planning time (fftw_execute) */
    double *cplx_arr;
    double *scratch;  /* c2r: working copy, so the input stays intact */
};

static fftw_plan mk_plan(int dir, int nx, int ny, int nz, double *r, double *c)
{
    struct ih_ref_fftw_plan_s *p = calloc(1, sizeof *p);
    if (!p) shim_fail("out of memory (plan)");
    if (nx < 1 || ny < 1 || nz < 2 || iho_fft3_init(&p->F, nx, ny, nz) != 0)
        shim_fail("unsupported transform size (needs an even last extent of 2^a 3^b 5^c)");
    p->dir = dir;
    p->nreal = (size_t)nx * ny * nz;
    p->ncomplex = (size_t)nx * ny * (nz / 2 + 1);
    p->real_arr = r;
    p->cplx_arr = c;
    if (dir == FFTW_BACKWARD) {
        p->scratch = malloc(sizeof(double) * 2 * p->ncomplex);
        if (!p->scratch) shim_fail("out of memory (plan scratch)");
    }
    return p;
}

fftw_plan fftw_plan_dft_r2c_1d(int n0, double *in, fftw_complex *out, unsigned flags)
{
    (void)flags;
    return mk_plan(FFTW_FORWARD, 1, 1, n0, in, (double *)out);
}

fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out, unsigned flags)
{
    (void)flags;
    return mk_plan(FFTW_FORWARD, 1, n0, n1, in, (double *)out);
}

fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in, fftw_complex *out,
                               unsigned flags)
{
    (void)flags;
    return mk_plan(FFTW_FORWARD, n0, n1, n2, in, (double *)out);
}

fftw_plan fftw_plan_dft_c2r_1d(int n0, fftw_complex *in, double *out, unsigned flags)
{
    (void)flags;
    return mk_plan(FFTW_BACKWARD, 1, 1, n0, out, (double *)in);
}

fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex *in, double *out, unsigned flags)
{
    (void)flags;
    return mk_plan(FFTW_BACKWARD, 1, n0, n1, out, (double *)in);
}

fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in, double *out,
                               unsigned flags)
{
    (void)flags;
    return mk_plan(FFTW_BACKWARD, n0, n1, n2, out, (double *)in);
}

static void run_r2c(const fftw_plan p, const double *in, double *out)
{
    if (p->dir != FFTW_FORWARD) shim_fail("r2c execution of a c2r plan");
    iho_fft3_r2c(&p->F, in, out);
}

static void run_c2r(const fftw_plan p, const double *in, double *out)
{
    if (p->dir != FFTW_BACKWARD) shim_fail("c2r execution of an r2c plan");
    memcpy(p->scratch, in, sizeof(double) * 2 * p->ncomplex);
    iho_fft3_c2r(&p->F, p->scratch, out);
}

void fftw_execute(const fftw_plan p)
{
    if (p->dir == FFTW_FORWARD) run_r2c(p, p->real_arr, p->cplx_arr);
    else run_c2r(p, p->cplx_arr, p->real_arr);
}

void fftw_execute_dft_r2c(const fftw_plan p, double *in, fftw_complex *out)
{
    run_r2c(p, in, (double *)out);
}

void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex *in, double *out)
{
    run_c2r(p, (const double *)in, out);
}

void fftw_destroy_plan(fftw_plan p)
{
    if (!p) return;
    iho_fft3_free(&p->F);
    free(p->scratch);
    free(p);
}

void *fftw_malloc(size_t n)
{
    void *p = NULL;
    if (posix_memalign(&p, 64, n ? n : 1) != 0) return NULL;
    return p;
}

void fftw_free(void *p) { free(p); }

int fftw_alignment_of(double *p) { return (int)((uintptr_t)p % 16u); }

int fftw_init_threads(void) { return 1; }

void fftw_plan_with_nthreads(int nthreads) { (void)nthreads; /* OpenMP's count is used */ }

void fftw_cleanup_threads(void) {}

/* ------------------------------------------------------------------ HDF5 */

#define H5S_MAXRANK 4
#define ID_BASE ((hid_t)0x1000000)

enum { OBJ_FREE = 0, OBJ_FILE, OBJ_SPACE, OBJ_PLIST, OBJ_DSET, OBJ_TYPE };
enum { CLASS_DOUBLE = 0, CLASS_STRING = 1 };

typedef struct {
    char *name;
    int file;                    /* index into g_files */
    int tclass;
    size_t tsize;                /* string: fixed size in bytes */
    int rank;
    hsize_t dims[H5S_MAXRANK], maxdims[H5S_MAXRANK];
    unsigned char *data;         /* doubles (row-major) or string bytes */
    size_t nbytes;
} rec_dataset;

typedef struct {
    char *path;
    int writable;
    int open;
} rec_file;

typedef struct {
    int kind;
    int file;                    /* OBJ_FILE */
    int dset;                    /* OBJ_DSET: index into g_dsets */
    int rank;                    /* OBJ_SPACE */
    hsize_t dims[H5S_MAXRANK], maxdims[H5S_MAXRANK];
    int selected;
    hsize_t start[H5S_MAXRANK], count[H5S_MAXRANK];
    int layout;                  /* OBJ_PLIST */
    int tclass;                  /* OBJ_TYPE */
    size_t tsize;
} rec_obj;

static rec_obj *g_objs = NULL;
static size_t g_nobjs = 0, g_capobjs = 0;
static rec_dataset *g_dsets = NULL;
static size_t g_ndsets = 0, g_capdsets = 0;
static rec_file *g_files = NULL;
static size_t g_nfiles = 0, g_capfiles = 0;

static void *grow(void *arr, size_t *cap, size_t need, size_t elem)
{
    if (need <= *cap) return arr;
    size_t nc = *cap ? *cap * 2 : 64;
    while (nc < need) nc *= 2;
    void *p = realloc(arr, nc * elem);
    if (!p) shim_fail("out of memory (hdf5 recorder)");
    memset((char *)p + *cap * elem, 0, (nc - *cap) * elem);
    *cap = nc;
    return p;
}

static hid_t new_obj(int kind, rec_obj **out)
{
    size_t i;
    for (i = 0; i < g_nobjs; ++i)
        if (g_objs[i].kind == OBJ_FREE) break;
    if (i == g_nobjs) {
        g_objs = grow(g_objs, &g_capobjs, g_nobjs + 1, sizeof *g_objs);
        ++g_nobjs;
    }
    memset(&g_objs[i], 0, sizeof g_objs[i]);
    g_objs[i].kind = kind;
    *out = &g_objs[i];
    return ID_BASE + (hid_t)i;
}

static rec_obj *get_obj(hid_t id, int kind)
{
    if (id < ID_BASE || (size_t)(id - ID_BASE) >= g_nobjs) return NULL;
    rec_obj *o = &g_objs[id - ID_BASE];
    return o->kind == kind ? o : NULL;
}

static herr_t free_obj(hid_t id, int kind)
{
    rec_obj *o = get_obj(id, kind);
    if (!o) return -1;
    o->kind = OBJ_FREE;
    return 0;
}

static size_t elems(int rank, const hsize_t *dims)
{
    size_t n = 1;
    for (int i = 0; i < rank; ++i) n *= (size_t)dims[i];
    return n;
}

static int new_file(const char *path, int writable)
{
    g_files = grow(g_files, &g_capfiles, g_nfiles + 1, sizeof *g_files);
    rec_file *f = &g_files[g_nfiles];
    f->path = strdup(path);
    f->writable = writable;
    f->open = 1;
    return (int)g_nfiles++;
}

static int new_dataset(int file, const char *name)
{
    for (size_t i = 0; i < g_ndsets; ++i)
        if (g_dsets[i].file == file && g_dsets[i].name && strcmp(g_dsets[i].name, name) == 0)
            return -1; /* HDF5 refuses a second dataset of the same name */
    g_dsets = grow(g_dsets, &g_capdsets, g_ndsets + 1, sizeof *g_dsets);
    rec_dataset *d = &g_dsets[g_ndsets];
    memset(d, 0, sizeof *d);
    d->name = strdup(name);
    d->file = file;
    return (int)g_ndsets++;
}

static int find_dataset(int file, const char *name)
{
    for (size_t i = 0; i < g_ndsets; ++i)
        if (g_dsets[i].file == file && g_dsets[i].name && strcmp(g_dsets[i].name, name) == 0)
            return (int)i;
    return -1;
}

static int write_file(int file)
{
    rec_file *f = &g_files[file];
    if (!f->writable) return 0;
    FILE *out = fopen(f->path, "wb");
    if (!out) return -1;
    int ok = fwrite("IHH5REC1", 1, 8, out) == 8;
    for (size_t i = 0; ok && i < g_ndsets; ++i) {
        const rec_dataset *d = &g_dsets[i];
        if (d->file != file || !d->name) continue;
        uint32_t len = (uint32_t)strlen(d->name), cls = (uint32_t)d->tclass,
                 rank = (uint32_t)d->rank;
        uint64_t nb = d->nbytes;
        ok = fwrite(&len, 4, 1, out) == 1 && fwrite(d->name, 1, len, out) == len &&
             fwrite(&cls, 4, 1, out) == 1 && fwrite(&rank, 4, 1, out) == 1;
        for (int r = 0; ok && r < d->rank; ++r) {
            uint64_t v = d->dims[r];
            ok = fwrite(&v, 8, 1, out) == 1;
        }
        ok = ok && fwrite(&nb, 8, 1, out) == 1 && (nb == 0 || fwrite(d->data, 1, nb, out) == nb);
    }
    ok = (fclose(out) == 0) && ok;
    return ok ? 0 : -1;
}

static int load_file(int file)
{
    FILE *in = fopen(g_files[file].path, "rb");
    if (!in) return -1;
    char magic[8];
    if (fread(magic, 1, 8, in) != 8 || memcmp(magic, "IHH5REC1", 8) != 0) {
        fclose(in);
        return -1;
    }
    for (;;) {
        uint32_t len, cls, rank;
        if (fread(&len, 4, 1, in) != 1) break;
        char *name = malloc(len + 1);
        if (!name || fread(name, 1, len, in) != len) { free(name); fclose(in); return -1; }
        name[len] = 0;
        if (fread(&cls, 4, 1, in) != 1 || fread(&rank, 4, 1, in) != 1 || rank > H5S_MAXRANK) {
            free(name);
            fclose(in);
            return -1;
        }
        int di = new_dataset(file, name);
        free(name);
        if (di < 0) { fclose(in); return -1; }
        rec_dataset *d = &g_dsets[di];
        d->tclass = (int)cls;
        d->rank = (int)rank;
        for (uint32_t r = 0; r < rank; ++r) {
            uint64_t v;
            if (fread(&v, 8, 1, in) != 1) { fclose(in); return -1; }
            d->dims[r] = d->maxdims[r] = v;
        }
        uint64_t nb;
        if (fread(&nb, 8, 1, in) != 1) { fclose(in); return -1; }
        d->data = malloc(nb ? nb : 1);
        d->nbytes = nb;
        if (!d->data || (nb && fread(d->data, 1, nb, in) != nb)) { fclose(in); return -1; }
        if (cls == CLASS_STRING) d->tsize = nb;
    }
    fclose(in);
    return 0;
}

hid_t H5Fcreate(const char *name, unsigned flags, hid_t fcpl, hid_t fapl)
{
    (void)flags; (void)fcpl; (void)fapl;
    rec_obj *o;
    hid_t id = new_obj(OBJ_FILE, &o);
    o->file = new_file(name, 1);
    return id;
}

hid_t H5Fopen(const char *name, unsigned flags, hid_t fapl)
{
    (void)flags; (void)fapl;
    int f = new_file(name, 0);
    if (load_file(f) != 0) return -1;
    rec_obj *o;
    hid_t id = new_obj(OBJ_FILE, &o);
    o->file = f;
    return id;
}

herr_t H5Fflush(hid_t object, H5F_scope_t scope)
{
    (void)scope;
    rec_obj *o = get_obj(object, OBJ_FILE);
    return o ? write_file(o->file) : -1;
}

herr_t H5Fclose(hid_t file)
{
    rec_obj *o = get_obj(file, OBJ_FILE);
    if (!o) return -1;
    const int f = o->file;
    herr_t st = write_file(f);
    for (size_t i = 0; i < g_ndsets; ++i)
        if (g_dsets[i].file == f) {
            free(g_dsets[i].name);
            free(g_dsets[i].data);
            g_dsets[i].name = NULL;
            g_dsets[i].data = NULL;
            g_dsets[i].file = -1;
        }
    for (size_t i = 0; i < g_nobjs; ++i)
        if (g_objs[i].kind == OBJ_DSET && g_objs[i].file == f) g_objs[i].kind = OBJ_FREE;
    g_files[f].open = 0;
    free_obj(file, OBJ_FILE);
    return st;
}

ssize_t H5Fget_obj_ids(hid_t file, unsigned types, size_t max_objs, hid_t *obj_id_list)
{
    rec_obj *o = get_obj(file, OBJ_FILE);
    if (!o) return -1;
    size_t n = 0;
    if (types & H5F_OBJ_DATASET)
        for (size_t i = 0; i < g_nobjs && n < max_objs; ++i)
            if (g_objs[i].kind == OBJ_DSET && g_objs[i].file == o->file)
                obj_id_list[n++] = ID_BASE + (hid_t)i;
    return (ssize_t)n;
}

hid_t H5Screate_simple(int rank, const hsize_t dims[], const hsize_t maxdims[])
{
    if (rank < 0 || rank > H5S_MAXRANK) return -1;
    rec_obj *o;
    hid_t id = new_obj(OBJ_SPACE, &o);
    o->rank = rank;
    for (int i = 0; i < rank; ++i) {
        o->dims[i] = dims[i];
        o->maxdims[i] = maxdims ? maxdims[i] : dims[i];
    }
    return id;
}

herr_t H5Sclose(hid_t space) { return free_obj(space, OBJ_SPACE); }

int H5Sget_simple_extent_dims(hid_t space, hsize_t dims[], hsize_t maxdims[])
{
    rec_obj *o = get_obj(space, OBJ_SPACE);
    if (!o) return -1;
    for (int i = 0; i < o->rank; ++i) {
        if (dims) dims[i] = o->dims[i];
        if (maxdims) maxdims[i] = o->maxdims[i];
    }
    return o->rank;
}

int H5Sget_simple_extent_ndims(hid_t space)
{
    rec_obj *o = get_obj(space, OBJ_SPACE);
    return o ? o->rank : -1;
}

herr_t H5Sselect_hyperslab(hid_t space, H5S_seloper_t op, const hsize_t start[],
                           const hsize_t stride[], const hsize_t count[], const hsize_t block[])
{
    rec_obj *o = get_obj(space, OBJ_SPACE);
    if (!o || op != H5S_SELECT_SET) return -1;
    for (int i = 0; i < o->rank; ++i) {
        if ((stride && stride[i] != 1) || (block && block[i] != 1)) return -1;
        if (start[i] + count[i] > o->dims[i]) return -1;
        o->start[i] = start[i];
        o->count[i] = count[i];
    }
    o->selected = 1;
    return 0;
}

hid_t H5Pcreate(hid_t cls)
{
    if (cls != H5P_DATASET_CREATE) return -1;
    rec_obj *o;
    return new_obj(OBJ_PLIST, &o);
}

herr_t H5Pclose(hid_t plist) { return free_obj(plist, OBJ_PLIST); }

herr_t H5Pset_layout(hid_t plist, H5D_layout_t layout)
{
    rec_obj *o = get_obj(plist, OBJ_PLIST);
    if (!o) return -1;
    o->layout = (int)layout;
    return 0;
}

herr_t H5Pset_chunk(hid_t plist, int ndims, const hsize_t dim[])
{
    rec_obj *o = get_obj(plist, OBJ_PLIST);
    if (!o || ndims < 1) return -1;
    for (int i = 0; i < ndims; ++i)
        if (dim[i] == 0) return -1;
    o->layout = (int)H5D_CHUNKED;
    return 0;
}

static int type_class(hid_t type, size_t *size)
{
    if (type == H5T_NATIVE_DOUBLE) { *size = sizeof(double); return CLASS_DOUBLE; }
    if (type == H5T_C_S1 || type == H5T_FORTRAN_S1) { *size = 1; return CLASS_STRING; }
    rec_obj *o = get_obj(type, OBJ_TYPE);
    if (!o) return -1;
    *size = o->tsize;
    return o->tclass;
}

hid_t H5Dcreate(hid_t loc, const char *name, hid_t type, hid_t space, hid_t lcpl,
                hid_t dcpl, hid_t dapl)
{
    (void)lcpl; (void)dcpl; (void)dapl;
    rec_obj *fo = get_obj(loc, OBJ_FILE), *so = get_obj(space, OBJ_SPACE);
    size_t tsize;
    int cls = type_class(type, &tsize);
    if (!fo || !so || cls < 0) return -1;
    const int file = fo->file;
    int di = new_dataset(file, name);
    if (di < 0) return -1;
    rec_dataset *d = &g_dsets[di];
    d->tclass = cls;
    d->tsize = tsize;
    d->rank = so->rank;
    for (int i = 0; i < so->rank; ++i) {
        d->dims[i] = so->dims[i];
        d->maxdims[i] = so->maxdims[i];
    }
    d->nbytes = elems(d->rank, d->dims) * tsize;
    d->data = calloc(d->nbytes ? d->nbytes : 1, 1);
    if (!d->data) shim_fail("out of memory (dataset)");
    rec_obj *o;
    hid_t id = new_obj(OBJ_DSET, &o);
    o->file = file;
    o->dset = di;
    return id;
}

hid_t H5Dopen(hid_t loc, const char *name, hid_t dapl)
{
    (void)dapl;
    rec_obj *fo = get_obj(loc, OBJ_FILE);
    if (!fo) return -1;
    const int file = fo->file;
    int di = find_dataset(file, name);
    if (di < 0) return -1;
    rec_obj *o;
    hid_t id = new_obj(OBJ_DSET, &o);
    o->file = file;
    o->dset = di;
    return id;
}

herr_t H5Dclose(hid_t dset) { return free_obj(dset, OBJ_DSET); }

hid_t H5Dget_space(hid_t dset)
{
    rec_obj *o = get_obj(dset, OBJ_DSET);
    if (!o) return -1;
    const rec_dataset *d = &g_dsets[o->dset];
    return H5Screate_simple(d->rank, d->dims, d->maxdims);
}

herr_t H5Dset_extent(hid_t dset, const hsize_t size[])
{
    rec_obj *o = get_obj(dset, OBJ_DSET);
    if (!o) return -1;
    rec_dataset *d = &g_dsets[o->dset];
    if (d->tclass != CLASS_DOUBLE || d->rank < 1 || d->rank > 2) return -1;
    for (int i = 0; i < d->rank; ++i)
        if (d->maxdims[i] != H5S_UNLIMITED && size[i] > d->maxdims[i]) return -1;
    const size_t n0 = (size_t)size[0], n1 = d->rank == 2 ? (size_t)size[1] : 1;
    const size_t o0 = (size_t)d->dims[0], o1 = d->rank == 2 ? (size_t)d->dims[1] : 1;
    double *nd = calloc((n0 * n1) ? (n0 * n1) : 1, sizeof(double));
    if (!nd) shim_fail("out of memory (extent)");
    const double *od = (const double *)d->data;
    for (size_t i = 0; i < (n0 < o0 ? n0 : o0); ++i)
        for (size_t j = 0; j < (n1 < o1 ? n1 : o1); ++j) nd[i * n1 + j] = od[i * o1 + j];
    free(d->data);
    d->data = (unsigned char *)nd;
    d->nbytes = n0 * n1 * sizeof(double);
    d->dims[0] = size[0];
    if (d->rank == 2) d->dims[1] = size[1];
    return 0;
}

/* element offsets of a file-space selection, row-major; returns the count */
static size_t selection(const rec_dataset *d, hid_t file_space, size_t **offs)
{
    const rec_obj *s = file_space == H5S_ALL ? NULL : get_obj(file_space, OBJ_SPACE);
    if (file_space != H5S_ALL && (!s || s->rank != d->rank)) return (size_t)-1;
    hsize_t start[H5S_MAXRANK] = {0}, count[H5S_MAXRANK];
    for (int i = 0; i < d->rank; ++i) {
        const int sel = s && s->selected;
        start[i] = sel ? s->start[i] : 0;
        count[i] = sel ? s->count[i] : d->dims[i];
        if (start[i] + count[i] > d->dims[i]) return (size_t)-1;
    }
    const size_t n = elems(d->rank, count);
    *offs = malloc((n ? n : 1) * sizeof **offs);
    if (!*offs) shim_fail("out of memory (selection)");
    if (d->rank <= 1) {
        for (size_t i = 0; i < n; ++i) (*offs)[i] = (size_t)start[0] * (d->rank == 1) + i;
    } else {
        size_t k = 0;
        for (size_t i = 0; i < count[0]; ++i)
            for (size_t j = 0; j < count[1]; ++j)
                (*offs)[k++] = (size_t)(start[0] + i) * d->dims[1] + start[1] + j;
    }
    return n;
}

static size_t mem_offset(hid_t mem_space)
{
    /* the reference's memory spaces are whole arrays or a selection that
       starts at 0 (io.c:717-720) */
    const rec_obj *m = mem_space == H5S_ALL ? NULL : get_obj(mem_space, OBJ_SPACE);
    if (!m || !m->selected) return 0;
    return m->rank == 1 ? (size_t)m->start[0] : 0;
}

herr_t H5Dwrite(hid_t dset, hid_t mem_type, hid_t mem_space, hid_t file_space, hid_t xfer,
                const void *buf)
{
    (void)xfer;
    rec_obj *o = get_obj(dset, OBJ_DSET);
    if (!o) return -1;
    rec_dataset *d = &g_dsets[o->dset];
    size_t msize;
    const int mcls = type_class(mem_type, &msize);
    if (d->tclass == CLASS_STRING) {
        if (mcls != CLASS_STRING) return -1;
        const char *s = buf;
        size_t n = strnlen(s, msize);
        if (n > d->tsize) n = d->tsize;
        free(d->data);
        d->data = malloc(n ? n : 1);
        memcpy(d->data, s, n);
        d->nbytes = n;
        return 0;
    }
    if (mcls != CLASS_DOUBLE) return -1;
    size_t *offs = NULL;
    const size_t n = selection(d, file_space, &offs);
    if (n == (size_t)-1) return -1;
    const double *src = (const double *)buf + mem_offset(mem_space);
    double *dst = (double *)d->data;
    for (size_t i = 0; i < n; ++i) dst[offs[i]] = src[i];
    free(offs);
    return 0;
}

herr_t H5Dread(hid_t dset, hid_t mem_type, hid_t mem_space, hid_t file_space, hid_t xfer,
               void *buf)
{
    (void)xfer;
    rec_obj *o = get_obj(dset, OBJ_DSET);
    if (!o) return -1;
    const rec_dataset *d = &g_dsets[o->dset];
    size_t msize;
    if (d->tclass != CLASS_DOUBLE || type_class(mem_type, &msize) != CLASS_DOUBLE) return -1;
    size_t *offs = NULL;
    const size_t n = selection(d, file_space, &offs);
    if (n == (size_t)-1) return -1;
    double *dst = (double *)buf + mem_offset(mem_space);
    const double *src = (const double *)d->data;
    for (size_t i = 0; i < n; ++i) dst[i] = src[offs[i]];
    free(offs);
    return 0;
}

hid_t H5Tcopy(hid_t type)
{
    size_t size;
    int cls = type_class(type, &size);
    if (cls < 0) return -1;
    rec_obj *o;
    hid_t id = new_obj(OBJ_TYPE, &o);
    o->tclass = cls;
    o->tsize = size;
    return id;
}

herr_t H5Tset_size(hid_t type, size_t size)
{
    rec_obj *o = get_obj(type, OBJ_TYPE);
    if (!o || o->tclass != CLASS_STRING || size == 0) return -1;
    o->tsize = size;
    return 0;
}

herr_t H5Tclose(hid_t type) { return free_obj(type, OBJ_TYPE); }

/* ------------------------------------------------------------------- GSL */

#define MT_N 624
#define MT_M 397

struct gsl_rng {
    uint32_t mt[MT_N];
    int mti;
};

static const gsl_rng_type mt19937_type = {"mt19937", 0xffffffffUL, 0};
const gsl_rng_type *gsl_rng_mt19937 = &mt19937_type;

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T)
{
    if (T != gsl_rng_mt19937) shim_fail("only gsl_rng_mt19937 is provided");
    gsl_rng *r = calloc(1, sizeof *r);
    if (!r) shim_fail("out of memory (rng)");
    gsl_rng_set(r, 0);
    return r;
}

void gsl_rng_set(const gsl_rng *rc, unsigned long seed)
{
    gsl_rng *r = (gsl_rng *)rc;
    if (seed == 0) seed = 4357; /* GSL's documented default seed */
    r->mt[0] = (uint32_t)(seed & 0xffffffffUL);
    for (int i = 1; i < MT_N; ++i)
        r->mt[i] = (uint32_t)(1812433253UL * (r->mt[i - 1] ^ (r->mt[i - 1] >> 30)) + (uint32_t)i);
    r->mti = MT_N;
}

void gsl_rng_free(gsl_rng *r) { free(r); }

static uint32_t mt_twist(uint32_t hi, uint32_t lo, uint32_t far)
{
    const uint32_t y = (hi & 0x80000000u) | (lo & 0x7fffffffu);
    return far ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}

unsigned long gsl_rng_get(const gsl_rng *rc)
{
    gsl_rng *r = (gsl_rng *)rc;
    if (r->mti >= MT_N) {
        int k;
        for (k = 0; k < MT_N - MT_M; ++k) r->mt[k] = mt_twist(r->mt[k], r->mt[k + 1], r->mt[k + MT_M]);
        for (; k < MT_N - 1; ++k)
            r->mt[k] = mt_twist(r->mt[k], r->mt[k + 1], r->mt[k + MT_M - MT_N]);
        r->mt[MT_N - 1] = mt_twist(r->mt[MT_N - 1], r->mt[0], r->mt[MT_M - 1]);
        r->mti = 0;
    }
    uint32_t y = r->mt[r->mti++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

double gsl_rng_uniform(const gsl_rng *r) { return (double)gsl_rng_get(r) / 4294967296.0; }

static const gsl_interp_type cspline_type = {"cspline"};
const gsl_interp_type *gsl_interp_cspline = &cspline_type;

static void gsl_absent(const char *fn)
{
    fprintf(stderr, "reference shim: %s is not provided (GSL is not installed); "
            "use IC_FROM_DAT_FILE_* initial data\n", fn);
}

gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n)
{
    (void)n;
    return (gsl_integration_workspace *)malloc(1);
}

void gsl_integration_workspace_free(gsl_integration_workspace *w) { free(w); }

gsl_integration_qawo_table *gsl_integration_qawo_table_alloc(
    double omega, double L, enum gsl_integration_qawo_enum sine, size_t n)
{
    (void)omega; (void)L; (void)sine; (void)n;
    return (gsl_integration_qawo_table *)malloc(1);
}

int gsl_integration_qawo_table_set(gsl_integration_qawo_table *t, double omega, double L,
                                   enum gsl_integration_qawo_enum sine)
{
    (void)t; (void)omega; (void)L; (void)sine;
    return GSL_SUCCESS;
}

void gsl_integration_qawo_table_free(gsl_integration_qawo_table *t) { free(t); }

int gsl_integration_qagiu(gsl_function *f, double a, double epsabs, double epsrel,
                          size_t limit, gsl_integration_workspace *workspace,
                          double *result, double *abserr)
{
    (void)f; (void)a; (void)epsabs; (void)epsrel; (void)limit; (void)workspace;
    *result = *abserr = 0.0;
    gsl_absent("gsl_integration_qagiu");
    return GSL_EUNIMPL;
}

int gsl_integration_qawf(gsl_function *f, const double a, const double epsabs,
                         const size_t limit, gsl_integration_workspace *workspace,
                         gsl_integration_workspace *cycle_workspace,
                         gsl_integration_qawo_table *wf, double *result, double *abserr)
{
    (void)f; (void)a; (void)epsabs; (void)limit; (void)workspace; (void)cycle_workspace;
    (void)wf;
    *result = *abserr = 0.0;
    gsl_absent("gsl_integration_qawf");
    return GSL_EUNIMPL;
}

gsl_interp_accel *gsl_interp_accel_alloc(void) { return (gsl_interp_accel *)malloc(1); }

void gsl_interp_accel_free(gsl_interp_accel *a) { free(a); }

gsl_spline *gsl_spline_alloc(const gsl_interp_type *T, size_t size)
{
    (void)T; (void)size;
    return (gsl_spline *)malloc(1);
}

int gsl_spline_init(gsl_spline *spline, const double xa[], const double ya[], size_t size)
{
    (void)spline; (void)xa; (void)ya; (void)size;
    gsl_absent("gsl_spline_init");
    return GSL_EUNIMPL;
}

double gsl_spline_eval(const gsl_spline *spline, double x, gsl_interp_accel *a)
{
    (void)spline; (void)x; (void)a;
    gsl_absent("gsl_spline_eval");
    return 0.0;
}

void gsl_spline_free(gsl_spline *spline) { free(spline); }
