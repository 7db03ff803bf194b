// C entry points into the CPU-emulated reference build (TEST INFRASTRUCTURE
// ONLY).  Compiled together with the reference's own sources; drives its
// exported imaging path and its stage functions on host buffers.
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "isar_imaging_export.h"
#include "isar_main.cuh"

// process globals of isar_imaging_export.cpp:4-35
extern RadarParameters paras;
extern CUDAHandle handles;
extern cuComplex* d_data_proc;
extern cuComplex* d_data_cut;
extern double* d_velocity;
extern float* d_hamming;
extern cuComplex* d_hrrp;

namespace {
// Count-prefixed arrays: per array an int64 element count, then the elements.
template <class T>
void dump(FILE* f, const T* p, size_t n)
{
    const int64_t c = (int64_t)n;
    std::fwrite(&c, sizeof(c), 1, f);
    if (n) std::fwrite(p, sizeof(T), n, f);
}
}  // namespace

extern "C" {

// dataParsing (isar_imaging_export.cpp:48-66) through the reference's export
// on the .wbd files in dir.  Writes to out_path: int32 [frame_len,
// frame_num], dataN (double), turnAngle (float).
int ref_parse(const char* dir, int polar_type, int data_type, const char* out_path)
{
    vec1D_DBL dn;
    vec1D_FLT ta;
    int frame_len = 0, frame_num = 0;
    if (dataParsing(&dn, &ta, &frame_len, &frame_num, std::string(dir), polar_type, data_type) != 0) return -1;
    FILE* f = std::fopen(out_path, "wb");
    if (!f) return -2;
    const int32_t fl[2] = {frame_len, frame_num};
    dump(f, fl, 2);
    dump(f, dn.data(), dn.size());
    dump(f, ta.data(), ta.size());
    std::fclose(f);
    return 0;
}

// dataParsing, imagingMemInit and one dataExtracting
// (isar_imaging_export.cpp:69-119) through the reference's exports: the
// window of window_len pulses from window_head, every sampling_stride-th
// pulse.  Writes to out_path: dataWFileSn (int32), dataNOut (double),
// turnAngleOut (float), dataW (float I/Q pairs).
int ref_extract(const char* dir, int polar_type, int data_type, int window_len, int window_head, int sampling_stride,
                const char* out_path)
{
    vec1D_DBL dn;
    vec1D_FLT ta;
    int frame_len = 0, frame_num = 0;
    if (dataParsing(&dn, &ta, &frame_len, &frame_num, std::string(dir), polar_type, data_type) != 0) return -1;
    vec1D_FLT img;
    vec1D_INT sn;
    vec1D_DBL dn_out;
    vec1D_FLT ta_out;
    vec1D_COM_FLT dw;
    imagingMemInit(&img, &sn, &dn_out, &ta_out, &dw, window_len, frame_len, data_type, true, false);
    int imaging_stride = window_len;
    const int rc = dataExtracting(&sn, &dn_out, &ta_out, &dw, dn, ta, frame_len, frame_num, sampling_stride,
                                  window_head, window_len, imaging_stride, data_type);
    int out = rc == 0 ? 0 : -3;
    FILE* f = out == 0 ? std::fopen(out_path, "wb") : nullptr;
    if (out == 0 && !f) out = -2;
    if (f) {
        dump(f, sn.data(), sn.size());
        dump(f, dn_out.data(), dn_out.size());
        dump(f, ta_out.data(), ta_out.size());
        dump(f, reinterpret_cast<const float*>(dw.data()), 2 * dw.size());
        std::fclose(f);
    }
    imagingMemDest(data_type, true, false);
    return out;
}

// One frame through the reference.  echo: 2*M*N floats; velocity: M doubles.
// img: M*512 floats (isarMainSingle).  Optional checkpoints recorded by a
// second pass through the same stage functions in the order of
// ISAR_RD_Imaging_Main_Ku (isar_main.cu:33-142): ra = profiles after
// rangeAlignmentParallel (2*M*N floats), cut = after HRRPCenter + cutRangeProfile
// and fe = after fastEntropy (2*M*512 floats each).
int ref_frame(const float* echo, const double* velocity, int M, int N, long long band_width, long long fc,
              double Tp, long long Fs, int data_type, int hpc, int mtrc, float* img, float* ra, float* cut,
              float* fe)
{
    if (data_type != 2) return -1;
    vec1D_FLT img_v;
    vec1D_INT sn;
    vec1D_DBL dn;
    vec1D_FLT ta;
    vec1D_COM_FLT dw;
    const int window_len = M;
    const int frame_len = 4 * N + 256;   // STRETCH: range_num = (frame_len - 256) / 4
    const bool b_hpc = hpc != 0, b_hrrp = false, b_mtrc = mtrc != 0;
    imagingMemInit(&img_v, &sn, &dn, &ta, &dw, window_len, frame_len, data_type, b_hpc, b_hrrp);
    if (paras.echo_num != M || paras.range_num != N) return -2;
    paras.band_width = band_width;
    paras.fc = fc;
    paras.Tp = Tp;
    paras.Fs = Fs;
    const size_t mn = (size_t)M * N;
    std::memcpy(d_data_proc, echo, mn * sizeof(cuComplex));
    if (b_hpc) std::memcpy(d_velocity, velocity, M * sizeof(double));
    isarMainSingle(img, data_type, 0, 1, b_hrrp, b_hpc, b_mtrc);
    if (ra || cut || fe) {
        std::memcpy(d_data_proc, echo, mn * sizeof(cuComplex));
        if (b_hpc) highSpeedCompensation(d_data_proc, d_velocity, paras, handles);
        rangeAlignmentParallel(d_data_proc, d_hamming, paras, handles);
        if (ra) std::memcpy(ra, d_data_proc, mn * sizeof(cuComplex));
        HRRPCenter(d_data_proc, 30, paras, handles);
        cutRangeProfile(d_data_proc, d_data_cut, paras.range_num, paras.range_num_cut, paras.data_num_cut,
                        handles.handle);
        if (cut) std::memcpy(cut, d_data_cut, (size_t)M * 512 * sizeof(cuComplex));
        fastEntropy(d_data_cut, paras.echo_num, paras.range_num_cut, handles);
        if (fe) std::memcpy(fe, d_data_cut, (size_t)M * 512 * sizeof(cuComplex));
    }
    imagingMemDest(data_type, b_hpc, b_hrrp);
    return 0;
}

// getHRRP (common.cu:541-580) on an M x N frame through the reference's
// imagingMemInit state (if_hrrp = true allocates d_hrrp): echo and out are
// 2*M*N floats.
int ref_hrrp(const float* echo, int M, int N, int data_type, float* out)
{
    vec1D_FLT img_v;
    vec1D_INT sn;
    vec1D_DBL dn;
    vec1D_FLT ta;
    vec1D_COM_FLT dw;
    const int frame_len = 4 * N + 256;
    imagingMemInit(&img_v, &sn, &dn, &ta, &dw, M, frame_len, data_type, false, true);
    if (paras.echo_num != M || paras.range_num != N) return -2;
    std::memcpy(d_data_proc, echo, (size_t)M * N * sizeof(cuComplex));
    getHRRP(d_hrrp, d_data_proc, d_hamming, paras, static_cast<DATA_TYPE>(data_type), handles);
    std::memcpy(out, d_hrrp, (size_t)M * N * sizeof(cuComplex));
    imagingMemDest(data_type, false, true);
    return 0;
}

// One IFDS pulse through the reference's pulseCompression class, as
// multiThreadIFDS drives it (common.cu:583-604): iq = 2*iq_len floats (the
// int16 samples converted), out = 2*4096 floats (RANGE_NUM_IFDS_PC).
int ref_pulse_compress(const float* iq, int iq_len, double velocity, long long band_width, long long fc, double Tp,
                       long long Fs, float* out)
{
    RadarParameters p{};
    p.band_width = band_width;
    p.fc = fc;
    p.Tp = Tp;
    p.Fs = Fs;
    pulseCompression pc(nextPow2(iq_len), iq_len, RANGE_NUM_IFDS_PC, p);
    cuComplex* d_out = nullptr;
    if (cudaMalloc((void**)&d_out, sizeof(cuComplex) * RANGE_NUM_IFDS_PC) != cudaSuccess) return -1;
    pc.pulseCompressionbyFFT(d_out, reinterpret_cast<const std::complex<float>*>(iq), velocity);
    std::memcpy(out, d_out, sizeof(cuComplex) * RANGE_NUM_IFDS_PC);
    cudaFree(d_out);
    return 0;
}

}  // extern "C"
