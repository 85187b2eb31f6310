/*
 * cil_gsd.h - frame output of the colony step in the GSD 1.0 file format, HOOMD schema.
 *
 * Two layers, both behind plain C types:
 *
 *  1. cil_gsd_*: a GSD file writer. For the same sequence of calls it lays the file out byte
 *     for byte as the reference's vendored gsd.c does (gsd.h:110-152, gsd.c:200-818): a 256-byte
 *     header, an index of 32-byte entries that starts with 128 entries and doubles by moving to
 *     the end of the file, a 128-entry list of 64-byte chunk names, chunk data appended at the
 *     end of the file, index entries written when a frame ends. Files it writes open with
 *     gsd.c and with HOOMD's GSD readers.
 *
 *  2. cil_frame_*: the device-fed frame writer that replaces outputGSDFrame
 *     (OutputWriter.cpp:505-644) for one colony of a cil_handle. One kernel packs the colony's
 *     elements, in the reference element order (cell-major, back element first), into FP32
 *     frame arrays in HBM; an asynchronous copy on a second CUDA stream moves them into pinned
 *     host memory while the caller's next cil_step launches run; a host thread writes the
 *     chunks and ends the frame. Two frames can be in flight.
 */
#ifndef CIL_GSD_H
#define CIL_GSD_H

#include <stddef.h>
#include <stdint.h>

#include "cil_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Chunk element types (enum gsd_type, gsd.h:19-31). */
typedef enum cil_gsd_type {
  CIL_GSD_UINT8 = 1,
  CIL_GSD_UINT16 = 2,
  CIL_GSD_UINT32 = 3,
  CIL_GSD_UINT64 = 4,
  CIL_GSD_INT8 = 5,
  CIL_GSD_INT16 = 6,
  CIL_GSD_INT32 = 7,
  CIL_GSD_INT64 = 8,
  CIL_GSD_FLOAT = 9,
  CIL_GSD_DOUBLE = 10
} cil_gsd_type;

/* Version word major << 16 | minor (gsd_make_version, gsd.c:437-440). */
#define CIL_GSD_VERSION(major, minor) ((uint32_t)(major) << 16 | (uint32_t)(minor))

typedef struct cil_gsd_file cil_gsd_file;

/* Creates (truncating) the file and opens it for appending frames: gsd_create followed by
 * gsd_open(GSD_OPEN_APPEND), as initGSDOutput does (OutputWriter.cpp:619-621). application
 * and schema are truncated to 63 characters. CIL_ERR_IO if the file cannot be written. */
cil_status cil_gsd_create(const char *path, const char *application, const char *schema, uint32_t schema_version,
                          cil_gsd_file **out);

/* Appends one chunk of N rows x M columns to the current frame (gsd_write_chunk,
 * gsd.h:137-143). N, M > 0 and data != NULL, else CIL_ERR_CONFIG (gsd.c returns -2). The
 * name is truncated to 63 characters; a name beyond the 128 the name list holds gets the id
 * 65535, as in gsd.c. */
cil_status cil_gsd_write_chunk(cil_gsd_file *f, const char *name, int32_t type, uint64_t N, uint32_t M,
                               const void *data);

/* Ends the frame: writes its index entries and advances the frame counter (gsd_end_frame,
 * gsd.c:693-733). */
cil_status cil_gsd_end_frame(cil_gsd_file *f);

/* Frames ended so far (gsd_get_nframes). 0 for NULL. */
uint64_t cil_gsd_nframes(const cil_gsd_file *f);

/* Closes the file and frees the handle. Chunks of a frame that was not ended stay out of
 * the index, as with gsd_close. NULL is a no-op. */
cil_status cil_gsd_close(cil_gsd_file *f);

/* Last error message of the file handle (empty if none). */
void cil_gsd_last_error(const cil_gsd_file *f, char *buf, size_t len);

/* ------------------------------------------------------------------------------------- */

typedef struct cil_frame_writer cil_frame_writer;

typedef struct cil_frame_options {
  const char *cell_name;     /* colony.nameCells[type]; NULL = "A" */
  const char *elem_names[2]; /* element tags; particle type j is "<cell>_<tag j>"; NULL = "BACK", "FRONT" */
  double length_unit;        /* units.Length; 2D frames place element j at z = -0.01 j length_unit; 0 = 1 */
  double lz;                 /* box z written in 2D frames; 0 = the largest element diameter uploaded
                              * for the colony (lz2d = colony.getMaxSigma(), OutputWriter.cpp:715) */
  int32_t flags;             /* CIL_FRAME_* */
  int32_t pad;
} cil_frame_options;

/* Also write particles/types in the file's first frame when its step is not 0 (the reference
 * writes it only in a frame of step 0, OutputWriter.cpp:539). */
#define CIL_FRAME_TYPES_IN_FIRST 1

/* Creates the GSD file (application "CIL", schema "hoomd" 1.1, OutputWriter.cpp:619) and the
 * device and pinned staging of the writer for one colony of h, sized for the colony's
 * capacity (28 bytes per element, twice on the device and twice in pinned memory). It may be
 * called before the colony is uploaded, as the reference opens its output before the run
 * (initializeOutput). The writer must be closed before h is destroyed. */
cil_status cil_frame_open(cil_handle *h, int32_t colony, const char *path, const cil_frame_options *opt,
                          cil_frame_writer **out);

/* Queues one frame of the colony's current state (outputGSDFrame(fp, id, ts),
 * OutputWriter.cpp:640-644), labelled with `step` (< 0: the handle's step counter; the
 * reference's final-state file passes 0, OutputWriter.cpp:735). Returns once the pack kernel
 * and the device-to-host copy are enqueued; it waits on the host only while both staging
 * slots hold frames not yet on disk. Chunks, in the reference's order: configuration/step,
 * /dimensions (3), /box; particles/N; particles/types (step 0); particles/Z, /diameter,
 * /typeid (dividing or dying colony, or step 0); particles/charge (dividing colony: cellTRho,
 * which the two-element model leaves at -1, Colony.cpp:258); particles/position and
 * /velocity (FP32, positions shifted by half the box); particles/mass (the cell pressure,
 * 0: the two-element model's pressure writer cellCellForcePressure has no host body,
 * MD.cuh:397-399, and Colony.cpp:214 initialises it to 0). A colony without cells writes
 * the configuration chunks and particles/N only. *frame (may be NULL) receives the frame's
 * index in the file. I/O errors of earlier frames are returned here as CIL_ERR_IO. */
cil_status cil_frame_write(cil_frame_writer *w, int64_t step, int64_t *frame);

/* Blocks until every queued frame is in the file. */
cil_status cil_frame_flush(cil_frame_writer *w);

/* Flushes, closes the file and frees the writer. NULL is a no-op. */
cil_status cil_frame_close(cil_frame_writer *w);

/* Counters of the writer: frames queued and written, bytes copied from the device, the
 * host time spent inside cil_frame_write (enqueue, waits for a free slot included) and in
 * the writer thread (copy wait and file writes), and the device time of the pack kernels and
 * of the device-to-host copies (CUDA events, summed over the frames written). */
typedef struct cil_frame_stats {
  int64_t frames_queued;
  int64_t frames_written;
  int64_t d2h_bytes;
  int64_t file_bytes;
  double enqueue_ms;
  double slot_wait_ms;
  double write_ms;
  double pack_ms;
  double copy_ms;
} cil_frame_stats;

cil_status cil_frame_get_stats(const cil_frame_writer *w, cil_frame_stats *out);

/* Last error message of the writer (empty if none). */
void cil_frame_last_error(const cil_frame_writer *w, char *buf, size_t len);

#ifdef __cplusplus
}
#endif
#endif /* CIL_GSD_H */
