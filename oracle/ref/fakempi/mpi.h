/* A stand-in for the few MPI calls the reference's parallel tempering makes
 * (Faunus::MPI in include/faunus/mpi.h: MPI_Init, MPI_Comm_size/rank,
 * MPI_Finalize, MPI_Allreduce of doubles, MPI_Issend/MPI_Irecv/MPI_Wait of
 * doubles, MPI_Abort), so that the reference's own ParallelTempering
 * (move.h:6520-6771) can run where no MPI library is installed.
 *
 * Test infrastructure only (oracle/ref/ref_harness_pt.cpp). The ranks are
 * separate processes started by a launcher with FAKEMPI_RANK, FAKEMPI_SIZE
 * and FAKEMPI_DIR (a scratch folder) in their environment. A message is a
 * file in that folder, written under a temporary name and renamed into
 * place; the receiver polls for it, reads it and removes it. Every wait ends
 * after FAKEMPI_TIMEOUT seconds (default 120) with a message on stderr and
 * exit(3), so a rank whose partner died never hangs.
 *
 * Sends complete at once (the message is in the folder), which is
 * observationally the same for a program that waits on its sends after its
 * receives, as FloatTransmitter::swapf does. */
#pragma once
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include <unistd.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_SUM 1
#define MPI_SUCCESS 0

struct MPI_Status {
    int MPI_SOURCE, MPI_TAG, MPI_ERROR;
};
struct fakempi_request {
    int kind = 0;   // 0 done, 1 receive pending
    int peer = 0, tag = 0, count = 0;
    double *buf = nullptr;
};
typedef fakempi_request MPI_Request;

namespace fakempi {

struct State {
    int rank = 0, size = 1;
    std::string dir;
    double timeout = 120.0;
    std::vector<long> sent, received;   // per peer: messages so far
    long collectives = 0;
};
inline State &st() {
    static State s;
    return s;
}
inline std::string msg_path(int src, int dst, long seq) {
    return st().dir + "/m_" + std::to_string(src) + "_" + std::to_string(dst) + "_" + std::to_string(seq);
}
inline void write_file(const std::string &path, const void *data, size_t bytes) {
    const std::string tmp = path + ".tmp";
    FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f || std::fwrite(data, 1, bytes, f) != bytes) {
        std::fprintf(stderr, "fakempi: cannot write %s\n", tmp.c_str());
        std::exit(3);
    }
    std::fclose(f);
    std::rename(tmp.c_str(), path.c_str());
}
// Waits (bounded) for a file of exactly `bytes` bytes and reads it.
inline void read_file(const std::string &path, void *data, size_t bytes, bool remove) {
    const auto t0 = std::chrono::steady_clock::now();
    while (true) {
        FILE *f = std::fopen(path.c_str(), "rb");
        if (f) {
            const size_t got = std::fread(data, 1, bytes, f);
            std::fclose(f);
            if (got != bytes) {
                std::fprintf(stderr, "fakempi: %s has the wrong size\n", path.c_str());
                std::exit(3);
            }
            if (remove) std::remove(path.c_str());
            return;
        }
        if (std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > st().timeout) {
            std::fprintf(stderr, "fakempi: rank %d gave up waiting for %s\n", st().rank, path.c_str());
            std::exit(3);
        }
        std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
}

}  // namespace fakempi

inline int MPI_Init(int *, char ***) {
    fakempi::State &s = fakempi::st();
    const char *r = std::getenv("FAKEMPI_RANK"), *n = std::getenv("FAKEMPI_SIZE"), *d = std::getenv("FAKEMPI_DIR");
    if (!r || !n || !d) {
        std::fprintf(stderr, "fakempi: FAKEMPI_RANK, FAKEMPI_SIZE and FAKEMPI_DIR must be set\n");
        std::exit(3);
    }
    s.rank = std::atoi(r);
    s.size = std::atoi(n);
    s.dir = d;
    if (const char *t = std::getenv("FAKEMPI_TIMEOUT")) s.timeout = std::atof(t);
    s.sent.assign(s.size, 0);
    s.received.assign(s.size, 0);
    return MPI_SUCCESS;
}
inline int MPI_Finalize() { return MPI_SUCCESS; }
inline int MPI_Comm_size(MPI_Comm, int *n) {
    *n = fakempi::st().size;
    return MPI_SUCCESS;
}
inline int MPI_Comm_rank(MPI_Comm, int *r) {
    *r = fakempi::st().rank;
    return MPI_SUCCESS;
}
inline int MPI_Abort(MPI_Comm, int code) {
    std::fprintf(stderr, "fakempi: rank %d aborted (%d)\n", fakempi::st().rank, code);
    std::exit(code ? code : 3);
}
inline int MPI_Issend(const void *buf, int count, MPI_Datatype, int dst, int, MPI_Comm, MPI_Request *req) {
    fakempi::State &s = fakempi::st();
    fakempi::write_file(fakempi::msg_path(s.rank, dst, s.sent[dst]++), buf, (size_t)count * sizeof(double));
    req->kind = 0;
    return MPI_SUCCESS;
}
inline int MPI_Irecv(void *buf, int count, MPI_Datatype, int src, int tag, MPI_Comm, MPI_Request *req) {
    req->kind = 1;
    req->peer = src;
    req->tag = tag;
    req->count = count;
    req->buf = static_cast<double *>(buf);
    return MPI_SUCCESS;
}
inline int MPI_Wait(MPI_Request *req, MPI_Status *status) {
    fakempi::State &s = fakempi::st();
    if (req->kind == 1) {
        fakempi::read_file(fakempi::msg_path(req->peer, s.rank, s.received[req->peer]++), req->buf,
                           (size_t)req->count * sizeof(double), true);
        if (status) {
            status->MPI_SOURCE = req->peer;
            status->MPI_TAG = req->tag;
            status->MPI_ERROR = MPI_SUCCESS;
        }
    }
    req->kind = 0;
    return MPI_SUCCESS;
}
// Sum over ranks, added in rank order on every rank (the same bits on all).
inline int MPI_Allreduce(const void *in, void *out, int count, MPI_Datatype, MPI_Op, MPI_Comm) {
    fakempi::State &s = fakempi::st();
    const long seq = s.collectives++;
    const std::string mine = s.dir + "/c_" + std::to_string(seq) + "_" + std::to_string(s.rank);
    fakempi::write_file(mine, in, (size_t)count * sizeof(double));
    std::vector<double> acc(count, 0.0), v(count);
    for (int r = 0; r < s.size; r++) {
        fakempi::read_file(s.dir + "/c_" + std::to_string(seq) + "_" + std::to_string(r), v.data(),
                           (size_t)count * sizeof(double), false);
        for (int i = 0; i < count; i++) acc[i] += v[i];
    }
    std::memcpy(out, acc.data(), (size_t)count * sizeof(double));
    return MPI_SUCCESS;
}
