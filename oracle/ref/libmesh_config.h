/* Configuration header for compiling libMesh's quadrature, shape-function
 * and element sources in place (test infrastructure: oracle/_ref).  It stands
 * in for the header libMesh's configure script generates: a default real
 * double-precision 3-D build with AMR and periodic boundaries enabled, the
 * options under which those sources are compiled by default.  Only the
 * macros these sources read are set. */
#ifndef ORACLE_REF_LIBMESH_CONFIG_H
#define ORACLE_REF_LIBMESH_CONFIG_H
#define LIBMESH_DIM 3
#define LIBMESH_DEFAULT_SCALAR_TYPE double
#define LIBMESH_DEFAULT_DOUBLE_PRECISION 1
#define LIBMESH_USE_REAL_NUMBERS 1
#define LIBMESH_ENABLE_AMR 1
#define LIBMESH_ENABLE_PERIODIC 1
#define LIBMESH_ENABLE_SECOND_DERIVATIVES 1
#define LIBMESH_ENABLE_UNIQUE_ID 1
#define LIBMESH_DOF_ID_BYTES 4
#define LIBMESH_UNIQUE_ID_BYTES 8
#define LIBMESH_SUBDOMAIN_ID_BYTES 2
#define LIBMESH_PROCESSOR_ID_BYTES 2
#define LIBMESH_BOUNDARY_ID_BYTES 2
#define LIBMESH_HAVE_GETTIMEOFDAY 1
#define LIBMESH_HAVE_SYS_TIME_H 1
#define LIBMESH_HAVE_CXX17 1
#endif
