/*
 * Single-rank message-passing stand-in used ONLY to compile the Object-MD
 * reference sources into the CPU oracle (test infrastructure, never shipped).
 *
 * The reference's CommunicationHandler (src/omd/comhandler.cpp) talks to its
 * 26 spatial neighbours with persistent point-to-point requests.  On one rank
 * every neighbour is this rank itself: a request sent towards neighbour i uses
 * tag BASE+(26-i) and the matching receive from neighbour 26-i uses tag
 * BASE+(26-i) (comhandler.cpp:266-285, 511-539), so a receive is satisfied by
 * the send request carrying the same tag.  Collectives reduce over one rank
 * and therefore copy their input.  Datatype handles are their byte sizes.
 */
#ifndef OMDG_ORACLE_MPI_STANDIN_H
#define OMDG_ORACLE_MPI_STANDIN_H

#include <cstdio>
#include <cstdlib>
#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
struct MPI_Status { int bytes; };

struct omdg_standin_request {
    int is_recv;   /* 1 = receive, 0 = send, 2 = send already consumed */
    void* buf;
    size_t bytes;
    int tag;
};
typedef omdg_standin_request* MPI_Request;

#define MPI_COMM_WORLD 0
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_DOUBLE 8
#define MPI_SUM 0
#define MPI_MAX 1
#define MPI_MIN 2
#define MPI_MAX_PROCESSOR_NAME 64

inline int MPI_Init(int*, char***) { return 0; }
inline int MPI_Finalize() { return 0; }
inline int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return 0; }
inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
inline int MPI_Get_processor_name(char* name, int* len) {
    std::strcpy(name, "oracle");
    *len = 6;
    return 0;
}
inline int MPI_Barrier(MPI_Comm) { return 0; }
inline int MPI_Abort(MPI_Comm, int code) { std::exit(code); }
inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }

inline int MPI_Allreduce(void* in, void* out, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
    std::memcpy(out, in, (size_t)n * (size_t)t);
    return 0;
}
inline int MPI_Reduce(void* in, void* out, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
    std::memcpy(out, in, (size_t)n * (size_t)t);
    return 0;
}
inline int MPI_Gather(void* in, int n, MPI_Datatype t, void* out, int, MPI_Datatype, int, MPI_Comm) {
    std::memcpy(out, in, (size_t)n * (size_t)t);
    return 0;
}
inline int MPI_Allgather(void* in, int n, MPI_Datatype t, void* out, int, MPI_Datatype, MPI_Comm) {
    std::memcpy(out, in, (size_t)n * (size_t)t);
    return 0;
}

/* Blocking stream messages are only used between distinct ranks. */
inline int MPI_Send(void*, int, MPI_Datatype, int, int, MPI_Comm) { return 0; }
inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status* s) {
    if (s) s->bytes = 0;
    return 0;
}
inline int MPI_Get_count(MPI_Status* s, MPI_Datatype t, int* c) { *c = s->bytes / t; return 0; }

inline int MPI_Send_init(void* b, int n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request* r) {
    *r = new omdg_standin_request{0, b, (size_t)n * (size_t)t, tag};
    return 0;
}
inline int MPI_Recv_init(void* b, int n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request* r) {
    *r = new omdg_standin_request{1, b, (size_t)n * (size_t)t, tag};
    return 0;
}
inline int MPI_Startall(int n, MPI_Request* r) {
    for (int i = 0; i < n; i++) {
        if (r[i]->is_recv != 1) continue;
        int matched = 0;
        for (int j = 0; j < n && !matched; j++) {
            if (r[j]->is_recv == 0 && r[j]->tag == r[i]->tag) {
                size_t len = r[i]->bytes < r[j]->bytes ? r[i]->bytes : r[j]->bytes;
                std::memcpy(r[i]->buf, r[j]->buf, len);
                r[j]->is_recv = 2;
                matched = 1;
            }
        }
        if (!matched) {
            std::fprintf(stderr, "mpi stand-in: receive with tag %d has no matching send\n", r[i]->tag);
            std::abort();
        }
    }
    for (int i = 0; i < n; i++)
        if (r[i]->is_recv == 2) r[i]->is_recv = 0;
    return 0;
}
inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return 0; }
inline int MPI_Request_free(MPI_Request* r) {
    delete *r;
    *r = 0;
    return 0;
}

#endif
