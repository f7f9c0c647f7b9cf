/* Stand-in for the autoconf-generated config.h of breseq's build, written for the reference oracle:
 * only the package strings the sources print.  Test infrastructure. */
#ifndef BSQ_REF_CONFIG_H
#define BSQ_REF_CONFIG_H
#define PACKAGE_NAME "breseq"
#define PACKAGE_VERSION "0.50.0"
#define PACKAGE_STRING "breseq 0.50.0"
#define PACKAGE_URL "https://github.com/barricklab/breseq"
#define PACKAGE_BUGREPORT "https://github.com/barricklab/breseq/issues"
#define GITHUB_REVISION_STRING "reference-oracle"
#endif
