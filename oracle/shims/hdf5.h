/* hdf5.h -- empty: cpic's HDF5 output is compiled out (src/output.c:131-399).
 * TEST INFRASTRUCTURE ONLY. */
