/*
 * main.h - the reference's operator interface, kept signature-for-signature.
 *
 *   3D: static void NL_Means(unsigned char* GPU_input, float* GPU_result)
 *       (3DNLM/main.h:6).  Sizes, SS, NS and h come from config.h.
 *   2D: static void NL_Means(unsigned char* GPU_input, float* GPU_result, int W,
 *       int H, int sr_size, int nb_size, int IMAGE_SIZE_X, int IMAGE_SIZE_Y)
 *       (2D NLM/11x11/main.h:6).
 * Both take HOST buffers: a pre-padded unsigned char input (halo
 * (SS+NS-2)/2 on every side, x fastest) and a float output on the input's
 * 0..255 scale, and return when the output is written.  The reference returns
 * void and ignores errors; so do these (a failure prints one line to stderr
 * and leaves the output untouched).  nlm_last_error() in nlm.h has the reason.
 */
#ifndef _MAIN_H_
#define _MAIN_H_

class NLMeansProcessor {
public:
    static void NL_Means(unsigned char* GPU_input, float* GPU_result);
    // Parameter names differ from the reference's IMAGE_SIZE_X/IMAGE_SIZE_Y only
    // because those are config.h macros here; types and order are the same.
    static void NL_Means(unsigned char* GPU_input, float* GPU_result, int W, int H, int sr_size,
                         int nb_size, int image_size_x, int image_size_y);
};

#endif
