/* Hand-written stand-in for the autoconf-generated config.h that the
 * reference's Unix build expects (unix/povconfig/syspovconfig.h includes it
 * when HAVE_CONFIG_H is defined).  Only used to compile the unmodified
 * reference sources into oracle/_ref for parity checking. */
#ifndef POVORACLE_REF_CONFIG_H
#define POVORACLE_REF_CONFIG_H
#define HAVE_NAN 1
#define HAVE_STD_ISNAN 1
#define HAVE_INF 1
#define HAVE_STD_ISINF 1
#define HAVE_UNISTD_H 1
#define HAVE_SYS_RESOURCE_H 1
#define HAVE_SYS_TIME_H 1
#define HAVE_TIME_H 1
#define HAVE_SYS_WAIT_H 1
#define HAVE_CLOCK_GETTIME 1
#define HAVE_DECL_CLOCK_MONOTONIC 1
#define HAVE_DECL_CLOCK_REALTIME 1
#define HAVE_DECL_CLOCK_PROCESS_CPUTIME_ID 1
#define HAVE_DECL_CLOCK_THREAD_CPUTIME_ID 1
#define HAVE_GETRUSAGE 1
#define HAVE_DECL_RUSAGE_SELF 1
#define HAVE_DECL_RUSAGE_THREAD 1
#define HAVE_DECL_RUSAGE_LWP 0
#define HAVE_NANOSLEEP 1
#define HAVE_USLEEP 1
#define HAVE_USECONDS_T 1
#define HAVE_CLOCKID_T 1
#define HAVE_GETCWD 1
#define HAVE_READLINK 1
#define HAVE_GETTIMEOFDAY 1
#define HAVE_PTHREAD 1
#define PACKAGE "povray"
#define PACKAGE_NAME "POV-Ray"
#define PACKAGE_VERSION "3.8.0-alpha"
#define VERSION_BASE "3.8"
#define BUILD_ARCH "linux"
#define BUILT_FOR "linux"
#define COMPILER_VENDOR "gnu"
#define COMPILER_VERSION "g++"
#define CXXFLAGS "-O2"
#define BUILT_BY "oracle/refbuild"
#define BUILTIN_IO_RESTRICTIONS "disabled"
#define BUILTIN_XWIN_DISPLAY "disabled"
#define BUILTIN_IMG_FORMATS "gif tga iff ppm pgm hdr bmp"
#define MISSING_IMG_FORMATS "png jpeg tiff openexr"
#define IO_RESTRICTIONS_DISABLED 1
#define LIBPNG_MISSING 1
#define LIBJPEG_MISSING 1
#define LIBTIFF_MISSING 1
#define OPENEXR_MISSING 1
#endif
