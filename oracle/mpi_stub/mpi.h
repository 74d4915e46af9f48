/*
 * Single-rank stand-in for the MPI API, used only to compile the reference's
 * CPU solver headers (Local_code/level-set_MPI_{2D,3D}/include) into the
 * oracle library under oracle/_ref/.  Test infrastructure, not product code.
 *
 * Semantics with one rank:
 *   - MPI_Isend / MPI_Irecv post requests; MPI_Waitall matches every posted
 *     receive with the posted send of the same tag (a rank that sends to
 *     itself, which is what the reference's periodic Y exchange does at one
 *     rank: Local_code/level-set_MPI_3D/include/config.h:263-264) and copies.
 *   - Allreduce / Reduce / Gather / Gatherv copy the local contribution.
 *   - MPI_PROC_NULL peers are skipped by the reference itself.
 */
#ifndef LSGB_ORACLE_MPI_STUB_H
#define LSGB_ORACLE_MPI_STUB_H

#include <string.h>
#include <stdio.h>
#include <stdlib.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
typedef int MPI_Request;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_PROC_NULL (-2)
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MAX_ERROR_STRING 64
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)

struct lsgb_mpi_req_t {
    int is_send;
    void* buf;
    int bytes;
    int tag;
};

static inline int lsgb_mpi_type_size(MPI_Datatype t) { return t == MPI_DOUBLE ? 8 : 4; }

/* Request table shared by one translation unit (the oracle driver). */
static struct lsgb_mpi_req_t lsgb_mpi_reqs[16];
static int lsgb_mpi_nreq = 0;

static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Abort(MPI_Comm, int code) { fprintf(stderr, "MPI_Abort(%d)\n", code); abort(); return 0; }
static inline int MPI_Error_string(int, char* s, int* len) { s[0] = 0; *len = 0; return 0; }
static inline double MPI_Wtime() {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static inline int lsgb_mpi_post(int is_send, const void* buf, int count, MPI_Datatype t,
                                int peer, int tag, MPI_Request* req) {
    if (peer != 0) { fprintf(stderr, "mpi stub: peer %d with one rank\n", peer); abort(); }
    if (lsgb_mpi_nreq >= 16) { fprintf(stderr, "mpi stub: request table full\n"); abort(); }
    lsgb_mpi_reqs[lsgb_mpi_nreq].is_send = is_send;
    lsgb_mpi_reqs[lsgb_mpi_nreq].buf = (void*)buf;
    lsgb_mpi_reqs[lsgb_mpi_nreq].bytes = count * lsgb_mpi_type_size(t);
    lsgb_mpi_reqs[lsgb_mpi_nreq].tag = tag;
    *req = lsgb_mpi_nreq++;
    return 0;
}

static inline int MPI_Isend(const void* buf, int count, MPI_Datatype t, int peer, int tag,
                            MPI_Comm, MPI_Request* req) {
    return lsgb_mpi_post(1, buf, count, t, peer, tag, req);
}

static inline int MPI_Irecv(void* buf, int count, MPI_Datatype t, int peer, int tag,
                            MPI_Comm, MPI_Request* req) {
    return lsgb_mpi_post(0, buf, count, t, peer, tag, req);
}

static inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) {
    /* Every receive takes the bytes of the send with its tag.  Sends are
     * copied into a staging buffer first so that a receive that overlaps
     * another send's source region cannot corrupt it. */
    void* staged[16] = {0};
    for (int s = 0; s < lsgb_mpi_nreq; ++s) {
        if (!lsgb_mpi_reqs[s].is_send) continue;
        staged[s] = malloc((size_t)lsgb_mpi_reqs[s].bytes);
        memcpy(staged[s], lsgb_mpi_reqs[s].buf, (size_t)lsgb_mpi_reqs[s].bytes);
    }
    for (int r = 0; r < lsgb_mpi_nreq; ++r) {
        if (lsgb_mpi_reqs[r].is_send) continue;
        int found = 0;
        for (int s = 0; s < lsgb_mpi_nreq; ++s) {
            if (lsgb_mpi_reqs[s].is_send && lsgb_mpi_reqs[s].tag == lsgb_mpi_reqs[r].tag) {
                if (lsgb_mpi_reqs[s].bytes != lsgb_mpi_reqs[r].bytes) {
                    fprintf(stderr, "mpi stub: size mismatch\n"); abort();
                }
                memcpy(lsgb_mpi_reqs[r].buf, staged[s], (size_t)lsgb_mpi_reqs[r].bytes);
                found = 1;
                break;
            }
        }
        if (!found) { fprintf(stderr, "mpi stub: unmatched receive tag %d\n", lsgb_mpi_reqs[r].tag); abort(); }
    }
    for (int s = 0; s < 16; ++s) free(staged[s]);
    lsgb_mpi_nreq = 0;
    return 0;
}

static inline int MPI_Allreduce(const void* in, void* out, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
    memmove(out, in, (size_t)count * lsgb_mpi_type_size(t));
    return 0;
}
static inline int MPI_Reduce(const void* in, void* out, int count, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
    memmove(out, in, (size_t)count * lsgb_mpi_type_size(t));
    return 0;
}
static inline int MPI_Gather(const void* in, int count, MPI_Datatype t, void* out, int, MPI_Datatype,
                             int, MPI_Comm) {
    memmove(out, in, (size_t)count * lsgb_mpi_type_size(t));
    return 0;
}
static inline int MPI_Gatherv(const void* in, int count, MPI_Datatype t, void* out, const int*,
                              const int* displs, MPI_Datatype, int, MPI_Comm) {
    memmove((char*)out + (size_t)displs[0] * lsgb_mpi_type_size(t), in,
            (size_t)count * lsgb_mpi_type_size(t));
    return 0;
}

#endif
