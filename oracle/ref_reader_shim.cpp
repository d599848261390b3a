/*
 * The reference's problem-file reader, run on the CPU.  TEST INFRASTRUCTURE ONLY.
 *
 * This translation unit compiles the reference's own reader
 * (PSBA/readparams.cpp: readInitialSBAEstimate and its helpers) and its
 * input filter quat2vec (PSBA/misc.cpp) unmodified, as C++ with g++, by
 * mapping the MSVC-only CRT calls they use onto the standard ones
 * (fscanf_s / sscanf_s with numeric conversions only, which take no buffer
 * sizes, and fopen_s).  The sources are #included from where they lie (the
 * include path is given by oracle/build.py); nothing is copied into this
 * repository.  The built library lands in oracle/_ref/ and is used only to
 * pin this repository's reader (psba_gb300/io.py) against the reference's.
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

static inline int ref_fopen_s(FILE **fp, const char *name, const char *mode)
{
    *fp = std::fopen(name, mode);
    return *fp ? 0 : 1;
}
#define fopen_s ref_fopen_s
#define fscanf_s std::fscanf
#define sscanf_s std::sscanf

#include "readparams.cpp"
#include "misc.cpp"

extern "C" {

/* readInitialSBAEstimate with quat2vec as the input filter, as
 * PSBA/main.cpp:102-110 calls it.  The arrays are malloc'ed by the reader;
 * ref_reader_free releases them.  Returns 0. */
int ref_read_sba(const char *cams, const char *pts, int cnp, int filecnp, int *ncams, int *npts, int *nprojs,
                 double **motstruct, double **initrot, double **imgpts, double **cov, char **vmask)
{
    readInitialSBAEstimate((char *)cams, (char *)pts, cnp, 3, 2, quat2vec, filecnp, ncams, npts, nprojs, motstruct,
                           initrot, imgpts, cov, vmask);
    return 0;
}

void ref_reader_free(void *p) { std::free(p); }

}  // extern "C"
