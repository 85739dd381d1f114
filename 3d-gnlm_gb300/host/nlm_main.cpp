// Raw-array stand-in for the reference's OpenCV driver 3DNLM/nlm.cpp (OpenCV is
// not available, so images are raw bytes).  Steps kept from the reference:
//   1. read an 8-bit IMAGE_SIZE_Y x IMAGE_SIZE_X slice (nlm.cpp:31),
//   2. pad it by (SS+NS-2)/2 with BORDER_REFLECT_101 in x and y (nlm.cpp:36-41),
//   3. replicate the padded slice into depth+SS+NS-2 planes (nlm.cpp:55-61),
//   4. call NLMeansProcessor::NL_Means (nlm.cpp:65),
//   5. truncate float -> unsigned char (nlm.cpp:68-72),
//   6. write output.bin as int dim, int height, int width, uchar[] (nlm.cpp:17-24).
// Usage: nlm_legacy <input.raw> [output.bin] [--volume]
//   --volume: the input is a full depth x Y x X uchar volume (padded here in
//   z by REFLECT_101 as well) instead of one slice.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "config.h"
#include "main.h"

static int reflect101(int i, int n) {
    if (n <= 1) return 0;
    const int period = 2 * n - 2;
    i %= period;
    if (i < 0) i += period;
    return i < n ? i : period - i;
}

int main(int argc, char** argv) {
    if (argc < 2) {
        fprintf(stderr, "Usage: %s <input.raw> [output.bin] [--volume]\n", argv[0]);
        return 1;
    }
    const char* out_path = (argc >= 3 && strcmp(argv[2], "--volume") != 0) ? argv[2] : "output.bin";
    bool volume = false;
    for (int i = 2; i < argc; ++i) volume |= strcmp(argv[i], "--volume") == 0;
    const int X = IMAGE_SIZE_X, Y = IMAGE_SIZE_Y, Z = depth;
    const int pad = (SS + NS - 2) / 2;
    const int W = X + 2 * pad, Hh = Y + 2 * pad, D = Z + 2 * pad;
    const size_t nin = volume ? (size_t)X * Y * Z : (size_t)X * Y;
    std::vector<unsigned char> img(nin);
    FILE* f = fopen(argv[1], "rb");
    if (!f || fread(img.data(), 1, nin, f) != nin) {
        fprintf(stderr, "cannot read %zu bytes from %s\n", nin, argv[1]);
        if (f) fclose(f);
        return 1;
    }
    fclose(f);
    std::vector<unsigned char> padded((size_t)W * Hh * D);
    for (int d = 0; d < D; ++d) {
        const int sz = volume ? reflect101(d - pad, Z) : 0;
        for (int i = 0; i < Hh; ++i)
            for (int j = 0; j < W; ++j)
                padded[((size_t)d * Hh + i) * W + j] =
                    img[((size_t)sz * Y + reflect101(i - pad, Y)) * X + reflect101(j - pad, X)];
    }
    std::vector<float> result((size_t)X * Y * Z);
    NLMeansProcessor::NL_Means(padded.data(), result.data());
    std::vector<unsigned char> result_uc(result.size());
    for (size_t i = 0; i < result.size(); ++i) result_uc[i] = (unsigned char)result[i];
    FILE* o = fopen(out_path, "wb");
    if (!o) {
        fprintf(stderr, "cannot write %s\n", out_path);
        return 1;
    }
    int dim = Z, height = X, width = Y;  // the reference writes (dim, img_W=rows, img_H=cols)
    fwrite(&dim, sizeof(int), 1, o);
    fwrite(&height, sizeof(int), 1, o);
    fwrite(&width, sizeof(int), 1, o);
    fwrite(result_uc.data(), 1, result_uc.size(), o);
    fclose(o);
    return 0;
}
