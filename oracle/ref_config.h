/* Build configuration used to compile the unmodified CTSim sources into the
 * oracle/_ref reference binaries (see oracle/Makefile).  Hand-written: the
 * container has no autoconf.  No FFTW, no MPI, no graphics, no DICOM. */
#define HAVE_SSTREAM 1
#define HAVE_GETOPT_H 1
#define HAVE_GETOPT_LONG 1
#define HAVE_STRING_H 1
#define HAVE_STRINGS_H 1
#define HAVE_STDLIB_H 1
#define HAVE_STDINT_H 1
#define HAVE_INTTYPES_H 1
#define HAVE_UNISTD_H 1
#define HAVE_SYS_TIME_H 1
#define HAVE_SYS_TYPES_H 1
#define HAVE_SYS_STAT_H 1
#define HAVE_GETTIMEOFDAY 1
#define HAVE_MATH_H 1
#define HAVE_SNPRINTF 1
#define HAVE_VSNPRINTF 1
#define HAVE_STRTOD 1
#define HAVE_STRTOL 1
#define HAVE_TIME 1
#define HAVE_HTONL 1
#define HAVE_NETINET_IN_H 1
#define SIZEOF_LONG 8
#define SIZEOF_INT 4
#define SIZEOF_SHORT 2
#define SIZEOF_FLOAT 4
#define SIZEOF_DOUBLE 8
#define VERSION "5.2.0"
#define PACKAGE "ctsim"
