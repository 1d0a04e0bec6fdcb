/* Test stub: the HDF5 type names InstaHeat's main.h and io.h mention, for a
 * syntax-only compile of the drop-in layer against those headers (HDF5 is not
 * installed here). */
#ifndef IH_TEST_HDF5_STUB_H
#define IH_TEST_HDF5_STUB_H
typedef long long hid_t;
typedef unsigned long long hsize_t;
typedef int herr_t;
typedef enum { H5D_COMPACT, H5D_CONTIGUOUS, H5D_CHUNKED } H5D_layout_t;
#endif
