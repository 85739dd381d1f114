/*
 * config.h - compile-time configuration of the drop-in NLMeansProcessor shim.
 *
 * Same macros as the reference's 3DNLM/config.h:4-9 (SS search width, NS patch
 * width, IMAGE_SIZE_X/Y, depth), plus PARAMETER, the filtering parameter h that
 * the reference fixes in 3DNLM/main.cu:13 (10 on the 0..255 scale of its
 * unsigned char input).  Every macro may be overridden with -D, which replaces
 * the reference's practice of rewriting this file with sed (3DNLM/run.sh:13-19).
 * The defaults are the 64^3, search 7^3, patch 3^3 workload.
 */
#ifndef CONFIG_H
#define CONFIG_H

#ifndef SS
#define SS 7
#endif
#ifndef NS
#define NS 3
#endif

#ifndef IMAGE_SIZE_X
#define IMAGE_SIZE_X 64
#endif
#ifndef IMAGE_SIZE_Y
#define IMAGE_SIZE_Y 64
#endif
#ifndef depth
#define depth 64
#endif

#ifndef PARAMETER
#define PARAMETER 10
#endif

#endif
