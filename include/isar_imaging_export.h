/*
 * isar_imaging_export.h -- the seven exports of Junf137/isar_imaging_cuda
 * (isar_imaging/isar_imaging_export.h:37-130), provided by libisar_gb300.so
 * with the same names, signatures and call order (calling_dll.cpp:46-87):
 *
 *   gpuDevInit -> dataParsing -> imagingMemInit
 *     -> loop { dataExtracting -> isarMainSingle [-> writeFileFLT] }
 *   -> imagingMemDest
 *
 * Like the reference these are extern "C" (unmangled) but take C++ standard
 * library types, so the caller must use the same C++ standard library
 * (libstdc++).  The library owns the device memory as process-wide state;
 * the calls are not thread-safe.  void functions report failures on stdout
 * as the reference does; the reason of the last failure is also available
 * from isar_get_last_error() (isar_gb300.h).
 */
#ifndef ISAR_IMAGING_EXPORT_H_
#define ISAR_IMAGING_EXPORT_H_

#include <complex>
#include <string>
#include <vector>

#if defined(__GNUC__)
#define DLL_EXPORT_API __attribute__((visibility("default")))
#else
#define DLL_EXPORT_API
#endif

typedef std::vector<int> vec1D_INT;
typedef std::vector<std::vector<int>> vec2D_INT;
typedef std::vector<float> vec1D_FLT;
typedef std::vector<std::vector<float>> vec2D_FLT;
typedef std::vector<double> vec1D_DBL;
typedef std::vector<std::vector<double>> vec2D_DBL;
typedef std::vector<std::complex<float>> vec1D_COM_FLT;
typedef std::vector<std::vector<std::complex<float>>> vec2D_COM_FLT;

/* isar_imaging_export.h:37 -- selects the device with the most SMs; 0 on success. */
extern "C" DLL_EXPORT_API int gpuDevInit();

/* isar_imaging_export.h:54 -- parses the .wbd files of dir_path (file name
 * pattern by polar_type / data_type), reads the radar parameters of the first
 * frame and the navigation data of every frame.  dataN: [4 x frame_total]
 * (range m, velocity m/s, azimuth deg, pitching deg); turnAngle: per frame. */
extern "C" DLL_EXPORT_API int dataParsing(vec1D_DBL* dataN, vec1D_FLT* turnAngle, int* frame_len, int* frame_num,
                                          const std::string& dir_path, const int& polar_type, const int& data_type);

/* isar_imaging_export.h:73 -- selects the frames of one image window
 * (uniform sampling) and moves their echoes to the device, reusing the
 * rows that overlap the previous window. */
extern "C" DLL_EXPORT_API int dataExtracting(vec1D_INT* dataWFileSn, vec1D_DBL* dataNOut, vec1D_FLT* turnAngleOut,
                                             vec1D_COM_FLT* dataW, const vec1D_DBL& dataN, const vec1D_FLT& turnAngle,
                                             const int& frame_len, const int& frame_num, const int& sampling_stride,
                                             const int& window_head, const int& window_len, int& imaging_stride,
                                             const int& data_type);

/* isar_imaging_export.h:93 -- sizes the host vectors (img = window_len*512)
 * and allocates the device workspace. */
extern "C" DLL_EXPORT_API void imagingMemInit(vec1D_FLT* img, vec1D_INT* dataWFileSn, vec1D_DBL* dataNOut,
                                              vec1D_FLT* turnAngleOut, vec1D_COM_FLT* dataW, const int& window_len,
                                              const int& frame_len, const int& data_type, const bool& if_hpc,
                                              const bool& if_hrrp);

/* isar_imaging_export.h:108 -- images the current window into h_img
 * (window_len x 512 floats).  option_alignment / option_phase are accepted
 * and unused, as in the reference. */
extern "C" DLL_EXPORT_API void isarMainSingle(float* h_img, const int& data_type, const int& option_alignment,
                                              const int& option_phase, const bool& if_hrrp, const bool& if_hpc,
                                              const bool& if_mtrc);

/* isar_imaging_export.h:119 -- one value per line, 5 decimals. */
extern "C" DLL_EXPORT_API void writeFileFLT(const std::string& outFilePath, const float* data,
                                            const size_t& data_size);

/* isar_imaging_export.h:130 -- releases the device workspace. */
extern "C" DLL_EXPORT_API void imagingMemDest(const int& data_type, const bool& if_hpc, const bool& if_hrrp);

#endif /* ISAR_IMAGING_EXPORT_H_ */
