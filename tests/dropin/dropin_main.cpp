// Drop-in caller (test program): the call order of the reference's demo caller
// (calling_dll.cpp:46-87) against libisar_gb300.so through the seven
// reference exports.  Usage:
//   dropin_main <dir> <polar_type> <window_len> <n_windows> <imaging_stride> <hpc> <mtrc> <out_prefix>
//               [<data_type>: 2 STRETCH (default), 1 IFDS]
// Writes <out_prefix><i>.txt per window (writeFileFLT) and prints the parsed
// frame_len / frame_num.
//   dropin_main --parse-bin <dir> <polar_type> <data_type> <out.bin>
//   dropin_main --extract-bin <dir> <polar_type> <data_type> <window_len> <window_head> <sampling_stride> <out.bin>
// write what dataParsing (and one dataExtracting) return, as count-prefixed
// arrays (int64 count, then the elements): int32 [frame_len, frame_num],
// dataN, turnAngle; or dataWFileSn, dataNOut, turnAngleOut, dataW.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "isar_imaging_export.h"

template <class T>
static void dump(FILE* f, const T* p, size_t n)
{
    const int64_t c = (int64_t)n;
    std::fwrite(&c, sizeof(c), 1, f);
    if (n) std::fwrite(p, sizeof(T), n, f);
}

int main(int argc, char** argv)
{
    if (argc == 6 && std::string(argv[1]) == "--parse-bin") {
        vec1D_DBL dataN;
        vec1D_FLT turnAngle;
        int frame_len = 0, frame_num = 0;
        if (dataParsing(&dataN, &turnAngle, &frame_len, &frame_num, argv[2], std::atoi(argv[3]),
                        std::atoi(argv[4])) != EXIT_SUCCESS)
            return 4;
        FILE* f = std::fopen(argv[5], "wb");
        if (!f) return 7;
        const int32_t fl[2] = {frame_len, frame_num};
        dump(f, fl, 2);
        dump(f, dataN.data(), dataN.size());
        dump(f, turnAngle.data(), turnAngle.size());
        std::fclose(f);
        return 0;
    }
    if (argc == 9 && std::string(argv[1]) == "--extract-bin") {
        const int data_type = std::atoi(argv[4]), window_len = std::atoi(argv[5]);
        const int window_head = std::atoi(argv[6]), sampling_stride = std::atoi(argv[7]);
        vec1D_DBL dataN, dataNOut;
        vec1D_FLT turnAngle, turnAngleOut, img;
        vec1D_INT dataWFileSn;
        vec1D_COM_FLT dataW;
        int frame_len = 0, frame_num = 0;
        if (gpuDevInit() != EXIT_SUCCESS) return 3;
        if (dataParsing(&dataN, &turnAngle, &frame_len, &frame_num, argv[2], std::atoi(argv[3]), data_type) !=
            EXIT_SUCCESS)
            return 4;
        imagingMemInit(&img, &dataWFileSn, &dataNOut, &turnAngleOut, &dataW, window_len, frame_len, data_type, true,
                       false);
        int imaging_stride = window_len;
        if (dataExtracting(&dataWFileSn, &dataNOut, &turnAngleOut, &dataW, dataN, turnAngle, frame_len, frame_num,
                           sampling_stride, window_head, window_len, imaging_stride, data_type) != EXIT_SUCCESS)
            return 6;
        FILE* f = std::fopen(argv[8], "wb");
        if (!f) return 7;
        dump(f, dataWFileSn.data(), dataWFileSn.size());
        dump(f, dataNOut.data(), dataNOut.size());
        dump(f, turnAngleOut.data(), turnAngleOut.size());
        dump(f, reinterpret_cast<const float*>(dataW.data()), 2 * dataW.size());
        std::fclose(f);
        imagingMemDest(data_type, true, false);
        return 0;
    }
    if (argc == 4 && std::string(argv[1]) == "--parse") {
        // dataParsing only (no GPU needed): prints the parsed values
        vec1D_DBL dataN;
        vec1D_FLT turnAngle;
        int frame_len = 0, frame_num = 0;
        if (dataParsing(&dataN, &turnAngle, &frame_len, &frame_num, argv[2], std::atoi(argv[3]), 2) != EXIT_SUCCESS)
            return 4;
        std::printf("frame_len %d frame_num %d\n", frame_len, frame_num);
        const size_t total = dataN.size() / 4;
        for (size_t i = 0; i < total; ++i)
            std::printf("%zu %.6f %.6f %.6f %.6f %.6f\n", i, dataN[i], dataN[i + total], dataN[i + 2 * total],
                        dataN[i + 3 * total], turnAngle[i]);
        return 0;
    }
    if (argc < 9) {
        std::fprintf(stderr, "usage: %s dir polar window_len n_windows stride hpc mtrc out_prefix\n", argv[0]);
        return 2;
    }
    const std::string dir = argv[1];
    const int polar_type = std::atoi(argv[2]);
    const int window_len = std::atoi(argv[3]);
    const int n_windows = std::atoi(argv[4]);
    int imaging_stride = std::atoi(argv[5]);
    const bool if_hpc = std::atoi(argv[6]) != 0, if_mtrc = std::atoi(argv[7]) != 0, if_hrrp = false;
    const std::string out = argv[8];
    const int data_type = argc > 9 ? std::atoi(argv[9]) : 2;
    const int sampling_stride = 1, option_alignment = 0, option_phase = 1;
    int window_head = 0;

    vec1D_DBL dataN;
    vec1D_FLT turnAngle;
    int frame_len = 0, frame_num = 0;
    vec1D_INT dataWFileSn;
    vec1D_DBL dataNOut;
    vec1D_FLT turnAngleOut;
    vec1D_COM_FLT dataW;
    vec1D_FLT img;

    if (gpuDevInit() != EXIT_SUCCESS) return 3;
    if (dataParsing(&dataN, &turnAngle, &frame_len, &frame_num, dir, polar_type, data_type) != EXIT_SUCCESS) return 4;
    std::printf("frame_len %d frame_num %d\n", frame_len, frame_num);
    imagingMemInit(&img, &dataWFileSn, &dataNOut, &turnAngleOut, &dataW, window_len, frame_len, data_type, if_hpc,
                   if_hrrp);
    if (img.size() != (size_t)window_len * 512) return 5;
    for (int i = 0; i < n_windows; ++i) {
        if (dataExtracting(&dataWFileSn, &dataNOut, &turnAngleOut, &dataW, dataN, turnAngle, frame_len, frame_num,
                           sampling_stride, window_head, window_len, imaging_stride, data_type) != EXIT_SUCCESS)
            return 6;
        isarMainSingle(img.data(), data_type, option_alignment, option_phase, if_hrrp, if_hpc, if_mtrc);
        writeFileFLT(out + std::to_string(i) + ".txt", img.data(), img.size());
        window_head += imaging_stride;
    }
    imagingMemDest(data_type, if_hpc, if_hrrp);
    return 0;
}
