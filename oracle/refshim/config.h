/* config.h -- stand-in for the autotools output of the reference build, used
 * only to compile reference sources into oracle/_ref (test infrastructure).
 * The reference's CPU path is built without OpenMP, CUDA, Score-P or AVX. */
#ifndef G5_REFSHIM_CONFIG_H
#define G5_REFSHIM_CONFIG_H
#endif
