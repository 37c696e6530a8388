/*
 * gsq_quest.h -- the quest signed-distance C interface over libgsq.so.
 *
 * The reference exposes its signed distance to C and Fortran through a global
 * query object: the C++ functions of quest/interface/signed_distance.hpp:88-319
 * and the shroud-generated C layer over them,
 * quest/interface/c_fortran/wrapQUEST.h:84-129 (QUEST_signed_distance_*, which
 * the Fortran module wrapfquest.F binds with bind(C)).  libgsq.so exports the
 * same QUEST_signed_distance_* symbols with the same signatures (the serial
 * build's: init_serial / init_serial_bufferify), so a C or Fortran caller of
 * the reference relinks against libgsq.so unchanged.  The query runs on the
 * GPU through gsq_sdf (gsq.h).
 *
 * Behaviour kept from the reference (quest/interface/signed_distance.cpp):
 *   - options are set before init; setting one after init aborts, as do
 *     evaluate and get_mesh_bounds before init, null bounds buffers and
 *     set_dimension(dim != 3) (the reference's SLIC_ERROR aborts; these void
 *     and double functions have no status to return).  The message is printed
 *     on stderr and kept in gsq_last_error() first;
 *   - init returns 0, or -1 when the file cannot be read (the message is in
 *     gsq_last_error()); init while initialized returns -1, as the reference's
 *     release build does (read_stl_mesh refuses a non-null mesh,
 *     quest/interface/internal/QuestHelpers.cpp:293-298);
 *   - defaults: dimension 3, closed surface, signs computed; finalize destroys
 *     the query and keeps the options.
 * Differences: every execution space (CPU, OpenMP, GPU) runs the query on the
 * GPU, whose results equal the reference's SEQ ones bit for bit; the allocator
 * ID is stored and unused (no Umpire); shared memory needs MPI-3 in the
 * reference, so it is ignored with a warning, as the reference's non-MPI-3
 * build does; init also returns -1 when the GPU query cannot be created.
 */
#ifndef GSQ_QUEST_H_
#define GSQ_QUEST_H_

#include <stdint.h>

#include "gsq.h"

#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* axom::quest::SignedDistExec (wrapQUEST.h:33-38) */
enum QUEST_SignedDistExec
{
  QUEST_SignedDistExec_CPU = 0,
  QUEST_SignedDistExec_OpenMP = 1,
  QUEST_SignedDistExec_GPU = 2
};

/* signed_distance_init(file) (signed_distance.hpp:117; wrapQUEST.h:92): reads
 * an STL file (gsq_stl_read) and builds the query; 0 on success, -1 otherwise. */
int QUEST_signed_distance_init_serial(const char* file);
/* The Fortran entry (wrapQUEST.h:96): file is a blank-padded buffer of
 * SHT_file_len characters; trailing blanks are dropped. */
int QUEST_signed_distance_init_serial_bufferify(char* file, int SHT_file_len);
/* signed_distance_initialized (signed_distance.hpp:143; wrapQUEST.h:99) */
bool QUEST_signed_distance_initialized(void);
/* signed_distance_get_mesh_bounds (signed_distance.hpp:308; wrapQUEST.h:101):
 * lo, hi receive the min / max over the mesh nodes, 3 doubles each. */
void QUEST_signed_distance_get_mesh_bounds(double* lo, double* hi);
/* option setters, before init only (signed_distance.hpp:157-232; wrapQUEST.h:103-115) */
void QUEST_signed_distance_set_dimension(int dim);
void QUEST_signed_distance_set_closed_surface(bool status);
void QUEST_signed_distance_set_compute_signs(bool computeSign);
void QUEST_signed_distance_set_allocator(int allocatorID);
void QUEST_signed_distance_set_verbose(bool status);
void QUEST_signed_distance_use_shared_memory(bool status);
void QUEST_signed_distance_set_execution_space(int execSpace);
/* signed_distance_evaluate(x, y, z) (signed_distance.hpp:248; wrapQUEST.h:117) */
double QUEST_signed_distance_evaluate_0(double x, double y, double z);
/* signed_distance_evaluate(x, y, z, cp, n) (signed_distance.hpp:266;
 * wrapQUEST.h:119-127): also the closest point and the pseudo-normal. */
double QUEST_signed_distance_evaluate_1(double x, double y, double z, double* cp_x, double* cp_y, double* cp_z,
                                        double* n_x, double* n_y, double* n_z);
/* signed_distance_finalize (signed_distance.hpp:319; wrapQUEST.h:129) */
void QUEST_signed_distance_finalize(void);

/* The C++-only overloads of signed_distance.hpp, as C entry points that
 * include/gsq.hpp's gsq::quest::signed_distance_* functions call:
 *   signed_distance_init(const mint::Mesh*) (signed_distance.hpp:137): a
 *     triangle mesh as node coordinates and 3 node ids per cell (host or
 *     device arrays, copied); aborts when already initialized, as the
 *     reference does; 0, or -1 when the GPU query cannot be created;
 *   signed_distance_evaluate(x, y, z, n, phi) (signed_distance.hpp:290): n
 *     points as three coordinate arrays (host or device), phi alike; aborts
 *     before init or on a null array. */
int gsq_quest_init_mesh(const double* x, const double* y, const double* z, int32_t nnodes, const int32_t* tris,
                        int32_t ntris);
void gsq_quest_evaluate_points(const double* x, const double* y, const double* z, int32_t npoints, double* phi);
/* The precision form of the global query (GSQ_PRECISION_MIXED by default:
 * equal to FP64 bit for bit, and faster); before init only, like the other
 * options.  Returns 0, or -1 for an unknown form. */
int gsq_quest_set_precision(int32_t precision);
/* The gsq_sdf handle of the global query (NULL before init), for gsq_sdf_*
 * calls on it (gsq_sdf_eval with closest points and normals in bulk, a
 * stream, gsq_sdf_backward). */
int gsq_quest_handle(const gsq_sdf** sdf);

#ifdef __cplusplus
}
#endif

#endif /* GSQ_QUEST_H_ */
