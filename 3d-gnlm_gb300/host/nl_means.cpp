// NLMeansProcessor::NL_Means - the reference's operator interface on top of the
// C ABI, so the reference's own driver (3DNLM/nlm.cpp:65, 2D NLM/11x11/nlm.cpp:36)
// links against this library unchanged.
//
// Semantics kept from the reference (3DNLM/main.cu:7607-7680,
// 2D NLM/11x11/main.cu:472-539): host buffers in and out, pre-padded unsigned
// char input, float output on the 0..255 scale, h = PARAMETER, synchronous,
// void return.  Changed: one staging pass + one fused kernel instead of four
// kernel variants x RUNS; device buffers cached by the library instead of
// allocated and freed per call; errors reported on stderr instead of ignored.
#include <stdio.h>

#include "config.h"
#include "main.h"
#include "nlm.h"

void NLMeansProcessor::NL_Means(unsigned char* GPU_input, float* GPU_result) {
    const int sr = (SS - 1) / 2, pr = (NS - 1) / 2;
    const int rc = nlm3d_forward_host(GPU_input, NLM_U8, IMAGE_SIZE_X, IMAGE_SIZE_Y, depth, sr, pr,
                                      (float)PARAMETER, GPU_result, NLM_FLAG_PREPADDED);
    if (rc != NLM_OK) fprintf(stderr, "NL_Means (3D): %s\n", nlm_last_error());
}

void NLMeansProcessor::NL_Means(unsigned char* GPU_input, float* GPU_result, int W, int H,
                                int sr_size, int nb_size, int IMAGE_SIZE_X_, int IMAGE_SIZE_Y_) {
    const int sr = (sr_size - 1) / 2, pr = (nb_size - 1) / 2;
    const int Xp = IMAGE_SIZE_X_ + sr_size + nb_size - 2;
    const int Yp = IMAGE_SIZE_Y_ + sr_size + nb_size - 2;
    // The reference passes (rows, cols) of the padded image as (W, H) and uses
    // W as the row stride, which only works for square images; accept either
    // order of the padded extents.
    if (!((W == Xp && H == Yp) || (W == Yp && H == Xp))) {
        fprintf(stderr, "NL_Means (2D): padded size %dx%d does not match %dx%d + %d\n", W, H,
                IMAGE_SIZE_X_, IMAGE_SIZE_Y_, sr_size + nb_size - 2);
        return;
    }
    const int rc = nlm2d_forward_host(GPU_input, NLM_U8, IMAGE_SIZE_X_, IMAGE_SIZE_Y_, sr, pr,
                                      (float)PARAMETER, GPU_result, NLM_FLAG_PREPADDED);
    if (rc != NLM_OK) fprintf(stderr, "NL_Means (2D): %s\n", nlm_last_error());
}
