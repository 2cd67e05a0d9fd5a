/* htr_gb300 — restart files in the reference's HDF5 layout.
 *
 * A restart is a directory with one file per tile and a master file, as
 * HTR's HDF.dump / HDF.load write and read them
 * (src/Utils/hdf_helper.rg:933-966 dumpTile / MODULE.dump, :1198-1243
 * loadTile / MODULE.load, driven from src/prometeo.rg:1285-1297 and
 * :1000-1007):
 *
 *   "<lo.x>,<lo.y>,<lo.z>-<hi.x>,<hi.y>,<hi.z>.hdf"   (tileFilename,
 *        src/Utils/hdf_helper.rg:357-367): one dataset per restart field
 *        (IOVars, src/prometeo.rg:145-153: rho, pressure, temperature,
 *        MolarFracs, velocity, dudtBoundary, dTdtBoundary), shaped
 *        (z, y, x) over the tile's rectangle, a vector field stored as an
 *        HDF5 array of doubles per point (create, src/Utils/hdf_helper.rg:199-331);
 *   "master.hdf" (dumpMasterFile, src/Utils/hdf_helper.rg:845-931): the
 *        attributes IO_VERSION, baseIndexSpace, tilesNumber, timeStep,
 *        simTime, channelForcing, SpeciesNames, Versions and the dataset
 *        `partitions` (one rectangle per tile, shaped (tz, ty, tx)).
 *
 * The files are written and read without an HDF5 library, in the earliest
 * HDF5 file format, with the structures libhdf5 itself writes for this
 * content under default properties (superblock 0, symbol-table groups,
 * version-1 object headers, contiguous storage).  The
 * master file's virtual datasets (createVirtualDataset,
 * src/Utils/hdf_helper.rg:387-618), a convenience view for post-processing
 * that the reference's loader does not read, are not written.
 *
 * A view's fields are device pointers (as for every htr_rhs.h entry point)
 * unless `flags` has HTR_RESTART_HOST_VIEW.  Field data pass through pinned
 * staging buffers in slabs of z-planes (at most 64 MiB each), copies and
 * file I/O overlapped; each call returns when its data are in the file or
 * in the view (it synchronises `stream`).  Errors: HTR_ERR_ARGUMENT,
 * HTR_ERR_LAYOUT, HTR_ERR_IO, HTR_ERR_FORMAT (a file that is not HDF5, is
 * truncated, fails a metadata checksum, or lacks a field or has another
 * shape), HTR_ERR_UNSUPPORTED (chunked, compressed or virtual storage,
 * link or attribute heaps beyond one block), HTR_ERR_CUDA;
 * htr_last_error() tells which.  Files are read in the earliest format and
 * in the newer one (superblock 2/3, version-2 object headers, compact or
 * dense links and attributes).
 */
#ifndef HTR_RESTART_H
#define HTR_RESTART_H

#include "htr_rhs.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int64_t timeStep;      /* stored as a 32-bit integer, the reference's `int` */
  double simTime;
  double channelForcing; /* 0 when the file has none */
} htr_restart_info;

enum {
  HTR_RESTART_HOST_VIEW = 1, /* the view's fields are host pointers */
  HTR_RESTART_PROFILES = 2   /* also MolarFracs_profile, velocity_profile, temperature_profile */
};

/* "<dirname>/<lo.x>,<lo.y>,<lo.z>-<hi.x>,<hi.y>,<hi.z>.hdf" into `out`
 * (tileFilename, src/Utils/hdf_helper.rg:357-367). */
int htr_restart_tile_filename(const char *dirname, htr_rect3 tile, char *out, size_t capacity);

/* dumpTile (src/Utils/hdf_helper.rg:933-947): the restart fields of `tile`. */
int htr_restart_write_tile(const char *dirname, const htr_fluid_view *view, htr_rect3 tile, int nSpec,
                           int flags, htr_stream_t stream);

/* loadTile (src/Utils/hdf_helper.rg:1198-1210): fills the restart fields
 * of `tile` from its file. */
int htr_restart_read_tile(const char *dirname, const htr_fluid_view *view, htr_rect3 tile, int nSpec,
                          int flags, htr_stream_t stream);

/* dumpMasterFile (src/Utils/hdf_helper.rg:845-931) and the attribute
 * writers HDF.write.{timeStep,simTime,channelForcing,SpeciesNames,Versions}
 * (src/Utils/hdf_helper.rg:1245-1333, :1382-1431).  `partitions` holds
 * tiles[0]*tiles[1]*tiles[2] rectangles, x fastest.  `species_names`
 * (nSpec names, at most 20 characters) and `versions` (solver and Legion
 * version strings) may be null to leave those attributes out. */
int htr_restart_write_master(const char *dirname, const htr_restart_info *info, htr_rect3 bounds,
                             const int64_t tiles[3], const htr_rect3 *partitions, int nSpec,
                             const char *const *species_names, const char *const *versions);

/* checkMasterFile / MasterFileTiles / MasterFileColors and HDF.read.*
 * (src/Utils/hdf_helper.rg:968-1196, :1335-1378): the scalar attributes,
 * the base index space, the tile counts and (when `capacity` is at least
 * their number) the tiles' rectangles, x fastest. */
int htr_restart_read_master(const char *dirname, htr_restart_info *info, htr_rect3 *bounds, int64_t tiles[3],
                            htr_rect3 *partitions, int64_t capacity);

/* Inspection of any HDF5 file of the supported subset (the reader behind
 * the functions above).  A dataset or attribute is named by its path below
 * the root group; `dataset` null means an attribute of the root group. */
int htr_h5_dataset_shape(const char *path, const char *dataset, int *rank, int64_t dims[8],
                         int64_t *doubles_per_element);
int htr_h5_read_doubles(const char *path, const char *dataset, double *out, int64_t count);
int htr_h5_string_attribute(const char *path, const char *dataset, const char *name, int64_t index,
                            char *out, size_t capacity);

#ifdef __cplusplus
}
#endif

#endif /* HTR_RESTART_H */
