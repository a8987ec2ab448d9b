// Runtime of the MPI stand-in (mpi.h) and the per-rank thread count of the
// Kokkos stand-in (Kokkos_Core.hpp).  Test infrastructure: it lets the
// reference's unmodified src/ run here, its ranks as threads of one process.
#include "mpi.h"
#include "shim_runtime.h"

#include <fcntl.h>
#include <unistd.h>

#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include <omp.h>

struct imexref_type {
    int kind;     // 0 basic, 1 subarray, 2 contiguous
    size_t size;  // bytes of one element (basic)
    int ndims = 0, sizes[3] = {0, 0, 0}, subsizes[3] = {0, 0, 0}, starts[3] = {0, 0, 0}, order = 0;
    int count = 0;
    imexref_type* old = nullptr;
};

struct imexref_type imexref_int = {0, sizeof(int)};
struct imexref_type imexref_double = {0, sizeof(double)};
struct imexref_type imexref_float = {0, sizeof(float)};
struct imexref_type imexref_char = {0, 1};

namespace {

int g_size = 1;
int g_threads = 0;  // OpenMP threads per rank (0: all / ranks)
thread_local int t_rank = 0;

std::mutex g_mu;
std::condition_variable g_cv;

// barrier
int g_arrived = 0;
long g_generation = 0;

void barrier()
{
    std::unique_lock<std::mutex> lk(g_mu);
    const long gen = g_generation;
    if (++g_arrived == g_size) {
        g_arrived = 0;
        ++g_generation;
        g_cv.notify_all();
        return;
    }
    g_cv.wait(lk, [&] { return g_generation != gen; });
}

// collectives: each rank's contribution, combined in rank order
std::vector<std::vector<char>> g_contrib;

void combine(const std::vector<std::vector<char>>& parts, void* recv, int count, MPI_Datatype type, MPI_Op op)
{
    if (type != MPI_DOUBLE) throw std::runtime_error("shim MPI: reductions of MPI_DOUBLE only");
    double* out = static_cast<double*>(recv);
    std::memcpy(out, parts[0].data(), (size_t)count * sizeof(double));
    for (size_t r = 1; r < parts.size(); ++r) {
        const double* v = reinterpret_cast<const double*>(parts[r].data());
        for (int i = 0; i < count; ++i) {
            if (op == MPI_SUM) out[i] += v[i];
            else if (op == MPI_MAX) out[i] = v[i] > out[i] ? v[i] : out[i];
            else if (op == MPI_MIN) out[i] = v[i] < out[i] ? v[i] : out[i];
        }
    }
}

int reduce(const void* send, void* recv, int count, MPI_Datatype type, MPI_Op op, int root)
{
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if ((int)g_contrib.size() != g_size) g_contrib.assign((size_t)g_size, {});
        g_contrib[(size_t)t_rank].assign(static_cast<const char*>(send),
                                         static_cast<const char*>(send) + (size_t)count * type->size);
    }
    barrier();
    if (root < 0 || root == t_rank) combine(g_contrib, recv, count, type, op);
    barrier();
    return MPI_SUCCESS;
}

// point to point: messages buffered at the send, matched by (src, dst, tag)
std::map<std::tuple<int, int, int>, std::deque<std::vector<char>>> g_mail;

}  // namespace

struct imexref_request {
    bool recv;
    void* buf;
    size_t bytes;
    int src, tag;
};

void imexref_set_world(int size, int threads)
{
    g_size = size;
    g_threads = threads;
}

void imexref_set_rank(int rank) { t_rank = rank; }

int imexref_threads()
{
    if (g_threads > 0) return g_threads;
    const int t = omp_get_max_threads() / g_size;
    return t > 0 ? t : 1;
}

extern "C" {

int MPI_Init(int*, char***) { return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }

int MPI_Comm_size(MPI_Comm, int* size)
{
    *size = g_size;
    return MPI_SUCCESS;
}

int MPI_Comm_rank(MPI_Comm, int* rank)
{
    *rank = t_rank;
    return MPI_SUCCESS;
}

int MPI_Barrier(MPI_Comm)
{
    barrier();
    return MPI_SUCCESS;
}

double MPI_Wtime(void)
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype type, MPI_Op op, MPI_Comm)
{
    return reduce(send, recv, count, type, op, -1);
}

int MPI_Reduce(const void* send, void* recv, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm)
{
    return reduce(send, recv, count, type, op, root);
}

int MPI_Isend(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm, MPI_Request* req)
{
    const char* p = static_cast<const char*>(buf);
    {
        std::lock_guard<std::mutex> lk(g_mu);
        g_mail[std::make_tuple(t_rank, dest, tag)].emplace_back(p, p + (size_t)count * type->size);
    }
    g_cv.notify_all();
    *req = new imexref_request{false, nullptr, 0, dest, tag};
    return MPI_SUCCESS;
}

int MPI_Irecv(void* buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm, MPI_Request* req)
{
    *req = new imexref_request{true, buf, (size_t)count * type->size, source, tag};
    return MPI_SUCCESS;
}

int MPI_Waitall(int count, MPI_Request* reqs, MPI_Status*)
{
    for (int i = 0; i < count; ++i) {
        imexref_request* r = reqs[i];
        if (!r) continue;
        if (r->recv) {
            std::unique_lock<std::mutex> lk(g_mu);
            auto key = std::make_tuple(r->src, t_rank, r->tag);
            g_cv.wait(lk, [&] { return !g_mail[key].empty(); });
            std::vector<char> msg = std::move(g_mail[key].front());
            g_mail[key].pop_front();
            if (msg.size() != r->bytes) throw std::runtime_error("shim MPI: message size mismatch");
            std::memcpy(r->buf, msg.data(), msg.size());
        }
        delete r;
        reqs[i] = MPI_REQUEST_NULL;
    }
    return MPI_SUCCESS;
}

int MPI_Type_create_subarray(int ndims, const int* sizes, const int* subsizes, const int* starts, int order,
                             MPI_Datatype oldtype, MPI_Datatype* newtype)
{
    if (ndims != 3) throw std::runtime_error("shim MPI: 3-d subarrays only");
    auto* t = new imexref_type{1, oldtype->size};
    t->ndims = ndims;
    for (int d = 0; d < 3; ++d) {
        t->sizes[d] = sizes[d];
        t->subsizes[d] = subsizes[d];
        t->starts[d] = starts[d];
    }
    t->order = order;
    t->old = oldtype;
    *newtype = t;
    return MPI_SUCCESS;
}

int MPI_Type_contiguous(int count, MPI_Datatype oldtype, MPI_Datatype* newtype)
{
    auto* t = new imexref_type{2, oldtype->size};
    t->count = count;
    t->old = oldtype;
    *newtype = t;
    return MPI_SUCCESS;
}

int MPI_Type_commit(MPI_Datatype*) { return MPI_SUCCESS; }

}  // extern "C"

// ----------------------------------------------------------------- MPI-IO --

namespace {

struct SharedFile {
    int fd = -1;
    int users = 0;
};
std::map<std::string, std::shared_ptr<SharedFile>> g_files;

}  // namespace

struct imexref_file {
    std::shared_ptr<SharedFile> shared;
    std::string name;
    long long disp = 0;         // view displacement (bytes)
    MPI_Datatype etype = nullptr;     // nullptr: byte view
    MPI_Datatype filetype = nullptr;
    long long pos = 0;          // individual file pointer, in etypes (bytes without a view)
};

namespace {

void pwrite_all(int fd, const void* buf, size_t n, long long off)
{
    const char* p = static_cast<const char*>(buf);
    while (n) {
        const ssize_t w = pwrite(fd, p, n, (off_t)off);
        if (w <= 0) throw std::runtime_error("shim MPI-IO: write failed");
        p += w;
        n -= (size_t)w;
        off += w;
    }
}

}  // namespace

extern "C" {

int MPI_File_open(MPI_Comm, const char* name, int amode, MPI_Info, MPI_File* fh)
{
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto& sf = g_files[name];
        if (!sf) sf = std::make_shared<SharedFile>();
        if (sf->fd < 0) {
            // MPI_MODE_CREATE | MPI_MODE_WRONLY: create if missing, never truncate
            const int flags = ((amode & MPI_MODE_RDWR) ? O_RDWR : O_WRONLY) | ((amode & MPI_MODE_CREATE) ? O_CREAT : 0);
            sf->fd = open(name, flags, 0644);
            if (sf->fd < 0) return 1;
        }
        ++sf->users;
        *fh = new imexref_file{sf, name};
    }
    barrier();
    return MPI_SUCCESS;
}

int MPI_File_close(MPI_File* fh)
{
    barrier();
    {
        std::lock_guard<std::mutex> lk(g_mu);
        imexref_file* f = *fh;
        if (--f->shared->users == 0) {
            close(f->shared->fd);
            f->shared->fd = -1;
            g_files.erase(f->name);
        }
        delete f;
        *fh = nullptr;
    }
    return MPI_SUCCESS;
}

int MPI_File_seek(MPI_File fh, MPI_Offset offset, int)
{
    fh->pos = offset;
    return MPI_SUCCESS;
}

int MPI_File_write(MPI_File fh, const void* buf, int count, MPI_Datatype type, MPI_Status*)
{
    if (fh->etype) throw std::runtime_error("shim MPI-IO: independent writes before a view only");
    const size_t n = (size_t)count * type->size;
    pwrite_all(fh->shared->fd, buf, n, fh->pos);
    fh->pos += (long long)n;
    return MPI_SUCCESS;
}

int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype etype, MPI_Datatype filetype, const char*, MPI_Info)
{
    fh->disp = disp;
    fh->etype = etype;
    fh->filetype = filetype;
    fh->pos = 0;
    barrier();
    return MPI_SUCCESS;
}

// Element e of the view (in etypes) lies in tile e / n of the filetype's
// subarray (n = its element count), at the subarray position of e mod n;
// tiles follow each other at the global array's extent.
int MPI_File_write_all(MPI_File fh, const void* buf, int count, MPI_Datatype type, MPI_Status*)
{
    if (!fh->etype || type->size != fh->etype->size) throw std::runtime_error("shim MPI-IO: write_all needs a view");
    const imexref_type* sub = fh->filetype->kind == 2 ? fh->filetype->old : fh->filetype;
    if (sub->kind != 1 || sub->order != MPI_ORDER_FORTRAN)
        throw std::runtime_error("shim MPI-IO: views of Fortran-order subarrays only");
    const long long es = (long long)type->size;
    const long long g0 = sub->sizes[0], g1 = sub->sizes[1], g2 = sub->sizes[2];
    const long long s0 = sub->subsizes[0], s1 = sub->subsizes[1], s2 = sub->subsizes[2];
    const long long n = s0 * s1 * s2, extent = g0 * g1 * g2;
    const char* p = static_cast<const char*>(buf);
    long long e = fh->pos;
    const long long end = fh->pos + count;
    while (e < end) {
        const long long tile = e / n, w = e - tile * n;
        const long long i = w % s0, j = (w / s0) % s1, k = w / (s0 * s1);
        const long long run = std::min(s0 - i, end - e);  // contiguous along the first dimension
        const long long off = tile * extent + (sub->starts[0] + i) + (sub->starts[1] + j) * g0 +
                              (sub->starts[2] + k) * g0 * g1;
        pwrite_all(fh->shared->fd, p + (e - fh->pos) * es, (size_t)(run * es), fh->disp + off * es);
        e += run;
    }
    (void)s2;
    fh->pos = end;
    barrier();
    return MPI_SUCCESS;
}

}  // extern "C"
