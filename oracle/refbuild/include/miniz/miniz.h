/* Stand-in for the five miniz 3.1.1 zip-writer calls breseq's output.cpp makes (the HTML report
 * archive, which the reference oracle never writes): every call reports failure.  Test
 * infrastructure only. */
#ifndef BSQ_REF_MINIZ_H
#define BSQ_REF_MINIZ_H
#include <stddef.h>
typedef int mz_bool;
typedef unsigned int mz_uint;
typedef struct { int unused; } mz_zip_archive;
#define MZ_DEFAULT_COMPRESSION 6
static inline mz_bool mz_zip_writer_init_file(mz_zip_archive*, const char*, size_t) { return 0; }
static inline mz_bool mz_zip_writer_add_file(mz_zip_archive*, const char*, const char*, const void*, unsigned short, mz_uint) { return 0; }
static inline mz_bool mz_zip_writer_finalize_archive(mz_zip_archive*) { return 0; }
static inline mz_bool mz_zip_writer_end(mz_zip_archive*) { return 0; }
#endif
