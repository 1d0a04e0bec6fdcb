/*
 * hdf5.h (shim) -- the subset of HDF5's C API that nikikilbertus/InstaHeat's
 * src/io.c and main_template.h use, implemented as an in-memory recorder.
 *
 * TEST INFRASTRUCTURE ONLY.  It lets the reference's own io.c compile and run
 * unmodified as part of the second oracle (oracle/_ref); libhdf5 is not
 * installed here.  Every dataset io.c creates is kept in memory with its
 * rank, extent and contents (H5Dset_extent grows it, hyperslab writes fill
 * it).  H5Fclose writes the file as a flat record file ("IHH5REC1"; see
 * ih_ref_shim.c) that oracle/ref.py reads back; H5Fopen/H5Dread read such a
 * file, so the reference's IC_FROM_H5_FILE follow-up path (io.c:754-788)
 * works on the recorder's own output.
 *
 * Calls covered (io.c:47-303, 319-335, 349-353, 361-488, 640-828):
 * H5Fcreate/open/close/flush/get_obj_ids, H5Screate_simple/close/
 * get_simple_extent_dims/get_simple_extent_ndims/select_hyperslab,
 * H5Pcreate/close/set_layout/set_chunk, H5Dcreate/open/close/write/read/
 * get_space/set_extent, H5Tcopy/set_size/close.  Datatypes: native double
 * and fixed-size strings (the commit-hash and method datasets).
 */
#ifndef IH_REF_SHIM_HDF5_H
#define IH_REF_SHIM_HDF5_H

#include <stddef.h>
#include <stdint.h> /* HDF5's public header brings these in; toolbox.h relies on it */
#include <sys/types.h>

typedef int64_t hid_t;
typedef unsigned long long hsize_t;
typedef long long hssize_t;
typedef int herr_t;

typedef enum H5D_layout_t {
    H5D_LAYOUT_ERROR = -1,
    H5D_COMPACT = 0,
    H5D_CONTIGUOUS = 1,
    H5D_CHUNKED = 2,
    H5D_VIRTUAL = 3,
    H5D_NLAYOUTS = 4
} H5D_layout_t;

typedef enum H5S_seloper_t {
    H5S_SELECT_NOOP = -1,
    H5S_SELECT_SET = 0,
    H5S_SELECT_OR,
    H5S_SELECT_AND,
    H5S_SELECT_XOR,
    H5S_SELECT_NOTB,
    H5S_SELECT_NOTA,
    H5S_SELECT_APPEND,
    H5S_SELECT_PREPEND,
    H5S_SELECT_INVALID
} H5S_seloper_t;

typedef enum H5F_scope_t { H5F_SCOPE_LOCAL = 0, H5F_SCOPE_GLOBAL = 1 } H5F_scope_t;

#define H5P_DEFAULT ((hid_t)0)
#define H5S_ALL ((hid_t)0)
#define H5S_UNLIMITED ((hsize_t)(-1))

#define H5F_ACC_RDONLY (0x0000u)
#define H5F_ACC_RDWR (0x0001u)
#define H5F_ACC_TRUNC (0x0002u)
#define H5F_ACC_EXCL (0x0004u)

#define H5F_OBJ_FILE (0x0001u)
#define H5F_OBJ_DATASET (0x0002u)
#define H5F_OBJ_GROUP (0x0004u)
#define H5F_OBJ_DATATYPE (0x0008u)
#define H5F_OBJ_ATTR (0x0010u)
#define H5F_OBJ_ALL (0x001Fu)

/* predefined identifiers: property-list class and datatypes */
#define H5P_DATASET_CREATE ((hid_t)0x7f000001)
#define H5T_NATIVE_DOUBLE ((hid_t)0x7f000010)
#define H5T_C_S1 ((hid_t)0x7f000011)
#define H5T_FORTRAN_S1 ((hid_t)0x7f000012)

hid_t H5Fcreate(const char *name, unsigned flags, hid_t fcpl, hid_t fapl);
hid_t H5Fopen(const char *name, unsigned flags, hid_t fapl);
herr_t H5Fclose(hid_t file);
herr_t H5Fflush(hid_t object, H5F_scope_t scope);
ssize_t H5Fget_obj_ids(hid_t file, unsigned types, size_t max_objs, hid_t *obj_id_list);

hid_t H5Screate_simple(int rank, const hsize_t dims[], const hsize_t maxdims[]);
herr_t H5Sclose(hid_t space);
int H5Sget_simple_extent_dims(hid_t space, hsize_t dims[], hsize_t maxdims[]);
int H5Sget_simple_extent_ndims(hid_t space);
herr_t H5Sselect_hyperslab(hid_t space, H5S_seloper_t op, const hsize_t start[],
                           const hsize_t stride[], const hsize_t count[],
                           const hsize_t block[]);

hid_t H5Pcreate(hid_t cls);
herr_t H5Pclose(hid_t plist);
herr_t H5Pset_layout(hid_t plist, H5D_layout_t layout);
herr_t H5Pset_chunk(hid_t plist, int ndims, const hsize_t dim[]);

hid_t H5Dcreate(hid_t loc, const char *name, hid_t type, hid_t space, hid_t lcpl,
                hid_t dcpl, hid_t dapl);
hid_t H5Dopen(hid_t loc, const char *name, hid_t dapl);
herr_t H5Dclose(hid_t dset);
herr_t H5Dwrite(hid_t dset, hid_t mem_type, hid_t mem_space, hid_t file_space, hid_t xfer,
                const void *buf);
herr_t H5Dread(hid_t dset, hid_t mem_type, hid_t mem_space, hid_t file_space, hid_t xfer,
               void *buf);
hid_t H5Dget_space(hid_t dset);
herr_t H5Dset_extent(hid_t dset, const hsize_t size[]);

hid_t H5Tcopy(hid_t type);
herr_t H5Tset_size(hid_t type, size_t size);
herr_t H5Tclose(hid_t type);

#endif
