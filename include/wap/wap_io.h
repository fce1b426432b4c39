/* wap_io.h -- host-side file formats and scan tables of the warp-and-project
 * command line (no GPU needed for any call here).
 *
 * These are the inputs and outputs around the reference's hot path: the
 * projection stack and result volumes in Analyze 7.5 / NIfTI-1 as CImg reads
 * and writes them, TIFF projection stacks as CImg's libtiff loader reads them, the projection-angle text file PSART's constructor reads,
 * the z-split of a projection stack into per-projection images, and the
 * low-discrepancy angle generator of the reference's sampling scripts.
 * Every call returns WAP_OK or a WAP_E* status (wap.h).
 */
#ifndef WAP_WAP_IO_H
#define WAP_WAP_IO_H

#include <stddef.h>

#include "wap/wap.h"

#ifdef __cplusplus
extern "C" {
#endif

#define WAP_EIO 7 /* file missing, short or malformed */

/* Analyze 7.5 pair (name.hdr + name.img, either name may be given) or a
 * single-file NIfTI-1 (.nii), as CImg::load_analyze reads it
 * (CImg.h:47829-47955): dims = W, H, D, C (missing ones are 1); datatype is
 * the Analyze code (2 u8, 4 i16, 8 i32, 16 f32, 64 f64).  Big-endian files
 * (header size >= 4096 when read natively) are byte-swapped. */
WAP_API int wap_analyze_info(const char *path, int *dims4, int *datatype);

/* Loads the data as float, each value multiplied by the header's scale factor
 * (0 means 1), like CImg<float>::load_analyze.  count = capacity of h_out in
 * floats; must be at least W*H*D*C. */
WAP_API int wap_analyze_load(const char *path, float *h_out, size_t count);

/* Writes a float image the way CImg<float>::save_analyze does
 * (CImg.h:51715-51790): a 348-byte header (name.hdr) plus raw data
 * (name.img), or one 352-byte-header file for a .nii name; a name without an
 * extension gets .hdr/.img.  voxel_size may be NULL (spacing 1). */
WAP_API int wap_analyze_save(const char *path, const float *h_data, const int *dims4, const float *voxel_size);

/* A TIFF projection stack as CImg<float>::load_tiff reads it (CImg.h:47445-
 * 47700; the reference enables libtiff for its projection input,
 * WaP_Tomo.h:7-8): every page is one z slice, each sample cast to float with
 * no scaling.  dims4 = W, H, pages, samples per pixel; bits and
 * sample_format (1 unsigned, 2 signed, 3 IEEE) of the first page (any may be
 * NULL).  Read: classic little- or big-endian TIFF, strips or tiles, one
 * sample per pixel of 8/16/32/64 bits, no compression, PackBits, LZW or
 * Deflate (through the system's zlib), horizontal-differencing predictor;
 * anything else, and any malformed file, is WAP_EIO.  Pages wider or taller
 * than 2^20 pixels, or stacks of more than 2^33 samples, are WAP_ETOOBIG; a
 * failed host allocation is WAP_ENOMEM. */
WAP_API int wap_tiff_info(const char *path, int *dims4, int *bits, int *sample_format);
/* Loads all pages, page after page (x fastest), into h_out (count >= W*H*pages floats). */
WAP_API int wap_tiff_load(const char *path, float *h_out, size_t count);

/* Reads up to n whitespace-separated angles (degrees) the way PSART's
 * constructor does (WaP_Tomo.cpp:324-331, `stream >> inputdegree[i]`):
 * reading stops at the first value that does not parse, and the entries not
 * read are set to 0 (the reference's zero-initialised global array).  Returns
 * the count read in *h_read (may be NULL); a missing file is WAP_EIO. */
WAP_API int wap_read_angles(const char *path, double *h_out, int n, int *h_read);

/* CImg::get_split('z', nb) of a stack of `depth` slices into nb pieces
 * (CImg.h:31389-31431, error-diffusion piece sizes): h_first[k] and
 * h_count[k] are the first slice and slice count of piece k.  PSART takes
 * piece k as projection k (WaP_Tomo.cpp:339), and the projector reads its
 * first slice. */
WAP_API int wap_split_z(int depth, int nb, int *h_first, int *h_count);

/* Low-discrepancy scanning angles (van der Corput radical inverse in base p,
 * Ns circle segments, a 0-degree projection inserted before every Nz-th;
 * Sampling_Model/low discrepancy sequence/Low_discrepency_squence.m:15-45).
 * Writes np angles in degrees. */
WAP_API int wap_lds_angles(int np, int ns, int p, int nz, double *h_out);

#ifdef __cplusplus
}
#endif
#endif /* WAP_WAP_IO_H */
