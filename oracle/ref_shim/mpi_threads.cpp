/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Thread-backed implementation of the MPI subset declared in mpi.h.  Ranks are
 * threads of one process.  Every collective runs in two barrier-separated
 * phases: each rank publishes its arguments, then each rank performs its own
 * share of the copy (or rank-ordered sum) by reading the other ranks' buffers,
 * and a second barrier keeps every buffer alive until all ranks are done.
 */
#include "mpi.h"

#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <vector>

namespace {

struct Block {
    size_t off, len;
};

struct TypeInfo {
    std::vector<Block> blocks;
    size_t extent;
    size_t align;
    bool contiguous;
};

struct Slot {
    const void* sbuf;
    void* rbuf;
    int scount;
    int rcount;
    const int* counts;
    const int* displs;
    MPI_Datatype type;
};

struct Msg {
    int src, dst, tag;
    std::vector<unsigned char> data;
};

struct World {
    int size = 1;
    std::mutex mu;
    std::condition_variable cv;
    int arrived = 0;
    unsigned long generation = 0;
    std::vector<Slot> slot{ Slot() };
    std::deque<Msg> box;
    std::deque<TypeInfo> types; /* deque: references stay valid while ranks add types */

    World()
    {
        types.push_back(TypeInfo{ {}, 0, 1, true });                 /* handle 0: invalid */
        types.push_back(TypeInfo{ { { 0, 4 } }, 4, 4, true });       /* MPI_INT */
        types.push_back(TypeInfo{ { { 0, 8 } }, 8, 8, true });       /* MPI_DOUBLE */
    }
};

World& world()
{
    static World w;
    return w;
}

thread_local int tl_rank = 0;

[[noreturn]] void die(const char* what)
{
    std::fprintf(stderr, "ref_shim mpi: %s\n", what);
    std::abort();
}

const TypeInfo& type_of(MPI_Datatype t)
{
    World& w = world();
    std::lock_guard<std::mutex> lk(w.mu);
    if (t <= 0 || (size_t)t >= w.types.size()) die("unknown datatype");
    return w.types[(size_t)t];
}

void copy_elems(void* dst, const void* src, int count, MPI_Datatype t)
{
    if (count <= 0 || dst == src) return;
    const TypeInfo& ti = type_of(t);
    if (ti.contiguous) {
        std::memmove(dst, src, (size_t)count * ti.extent);
        return;
    }
    auto* d = static_cast<unsigned char*>(dst);
    auto* s = static_cast<const unsigned char*>(src);
    for (int k = 0; k < count; ++k)
        for (const Block& b : ti.blocks) std::memcpy(d + k * ti.extent + b.off, s + k * ti.extent + b.off, b.len);
}

void barrier()
{
    World& w = world();
    if (w.size == 1) return;
    std::unique_lock<std::mutex> lk(w.mu);
    unsigned long gen = w.generation;
    if (++w.arrived == w.size) {
        w.arrived = 0;
        ++w.generation;
        w.cv.notify_all();
    } else {
        w.cv.wait(lk, [&] { return w.generation != gen; });
    }
}

/* Phase 1 of a collective: publish this rank's arguments. */
void publish(const Slot& s)
{
    World& w = world();
    {
        std::lock_guard<std::mutex> lk(w.mu);
        w.slot[(size_t)tl_rank] = s;
    }
    barrier();
}

const Slot& slot_of(int rank) { return world().slot[(size_t)rank]; }

unsigned char* at(void* base, int displ, MPI_Datatype t)
{
    return static_cast<unsigned char*>(base) + (size_t)displ * type_of(t).extent;
}

const unsigned char* at(const void* base, int displ, MPI_Datatype t)
{
    return static_cast<const unsigned char*>(base) + (size_t)displ * type_of(t).extent;
}

} // namespace

extern "C" {

void ugmpi_init_world(int size)
{
    World& w = world();
    std::lock_guard<std::mutex> lk(w.mu);
    if (size < 1) size = 1;
    w.size = size;
    w.arrived = 0;
    w.slot.assign((size_t)size, Slot());
    w.box.clear();
}

void ugmpi_set_rank(int rank) { tl_rank = rank; }

int MPI_Init(int*, char***) { return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }

int MPI_Comm_size(MPI_Comm, int* size)
{
    *size = world().size;
    return MPI_SUCCESS;
}

int MPI_Comm_rank(MPI_Comm, int* rank)
{
    *rank = tl_rank;
    return MPI_SUCCESS;
}

int MPI_Barrier(MPI_Comm)
{
    barrier();
    return MPI_SUCCESS;
}

int MPI_Bcast(void* buf, int count, MPI_Datatype type, int root, MPI_Comm)
{
    if (world().size == 1) return MPI_SUCCESS;
    publish(Slot{ buf, buf, count, count, nullptr, nullptr, type });
    if (tl_rank != root) copy_elems(buf, slot_of(root).sbuf, count, type);
    barrier();
    return MPI_SUCCESS;
}

int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op op, MPI_Comm)
{
    if (op != MPI_SUM || (type != MPI_INT && type != MPI_DOUBLE)) die("Allreduce: only MPI_SUM of MPI_INT/MPI_DOUBLE");
    World& w = world();
    if (w.size == 1) {
        copy_elems(recvbuf, sendbuf, count, type);
        return MPI_SUCCESS;
    }
    publish(Slot{ sendbuf, recvbuf, count, count, nullptr, nullptr, type });
    /* rank-ordered sums, so every rank gets the same bits whatever the thread timing */
    if (type == MPI_DOUBLE) {
        auto* r = static_cast<double*>(recvbuf);
        for (int k = 0; k < count; ++k) {
            double acc = static_cast<const double*>(slot_of(0).sbuf)[k];
            for (int q = 1; q < w.size; ++q) acc += static_cast<const double*>(slot_of(q).sbuf)[k];
            r[k] = acc;
        }
    } else {
        auto* r = static_cast<int*>(recvbuf);
        for (int k = 0; k < count; ++k) {
            int acc = static_cast<const int*>(slot_of(0).sbuf)[k];
            for (int q = 1; q < w.size; ++q) acc += static_cast<const int*>(slot_of(q).sbuf)[k];
            r[k] = acc;
        }
    }
    barrier();
    return MPI_SUCCESS;
}

int MPI_Allgather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
                  MPI_Datatype recvtype, MPI_Comm)
{
    World& w = world();
    if (w.size == 1) {
        copy_elems(recvbuf, sendbuf, sendcount, sendtype);
        return MPI_SUCCESS;
    }
    publish(Slot{ sendbuf, recvbuf, sendcount, recvcount, nullptr, nullptr, sendtype });
    for (int q = 0; q < w.size; ++q) copy_elems(at(recvbuf, q * recvcount, recvtype), slot_of(q).sbuf, recvcount, recvtype);
    barrier();
    return MPI_SUCCESS;
}

int MPI_Allgatherv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, const int* recvcounts,
                   const int* displs, MPI_Datatype recvtype, MPI_Comm)
{
    World& w = world();
    if (w.size == 1) {
        copy_elems(at(recvbuf, displs[0], recvtype), sendbuf, sendcount, sendtype);
        return MPI_SUCCESS;
    }
    publish(Slot{ sendbuf, recvbuf, sendcount, 0, recvcounts, displs, sendtype });
    for (int q = 0; q < w.size; ++q)
        copy_elems(at(recvbuf, displs[q], recvtype), slot_of(q).sbuf, recvcounts[q], recvtype);
    barrier();
    return MPI_SUCCESS;
}

int MPI_Gatherv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, const int* recvcounts,
                const int* displs, MPI_Datatype recvtype, int root, MPI_Comm)
{
    World& w = world();
    if (w.size == 1) {
        copy_elems(at(recvbuf, displs[0], recvtype), sendbuf, sendcount, sendtype);
        return MPI_SUCCESS;
    }
    publish(Slot{ sendbuf, recvbuf, sendcount, 0, recvcounts, displs, sendtype });
    if (tl_rank == root)
        for (int q = 0; q < w.size; ++q)
            copy_elems(at(recvbuf, displs[q], recvtype), slot_of(q).sbuf, recvcounts[q], recvtype);
    barrier();
    return MPI_SUCCESS;
}

int MPI_Scatterv(const void* sendbuf, const int* sendcounts, const int* displs, MPI_Datatype sendtype, void* recvbuf,
                 int recvcount, MPI_Datatype recvtype, int root, MPI_Comm)
{
    World& w = world();
    if (w.size == 1) {
        copy_elems(recvbuf, at(sendbuf, displs[0], sendtype), recvcount, recvtype);
        return MPI_SUCCESS;
    }
    /* only the root's counts and displacements are meaningful (the reference leaves the others unset) */
    publish(Slot{ sendbuf, recvbuf, 0, recvcount, tl_rank == root ? sendcounts : nullptr,
                  tl_rank == root ? displs : nullptr, sendtype });
    const Slot& r = slot_of(root);
    copy_elems(recvbuf, at(r.sbuf, r.displs[tl_rank], r.type), recvcount, recvtype);
    barrier();
    return MPI_SUCCESS;
}

int MPI_Send(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm)
{
    World& w = world();
    if (dest < 0 || dest >= w.size) die("Send: bad destination");
    const TypeInfo& ti = type_of(type);
    if (!ti.contiguous) die("Send: only contiguous types");
    Msg m{ tl_rank, dest, tag, {} };
    m.data.resize((size_t)count * ti.extent);
    if (!m.data.empty()) std::memcpy(m.data.data(), buf, m.data.size());
    {
        std::lock_guard<std::mutex> lk(w.mu);
        w.box.push_back(std::move(m));
    }
    w.cv.notify_all();
    return MPI_SUCCESS;
}

int MPI_Recv(void* buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm, MPI_Status* status)
{
    World& w = world();
    const TypeInfo& ti = type_of(type);
    std::unique_lock<std::mutex> lk(w.mu);
    for (;;) {
        for (auto it = w.box.begin(); it != w.box.end(); ++it) {
            if (it->dst == tl_rank && it->src == source && it->tag == tag) {
                size_t n = it->data.size();
                if (n > (size_t)count * ti.extent) die("Recv: message longer than the buffer");
                if (n) std::memcpy(buf, it->data.data(), n);
                if (status) {
                    status->MPI_SOURCE = source;
                    status->MPI_TAG = tag;
                    status->MPI_ERROR = MPI_SUCCESS;
                    status->bytes = (long)n;
                }
                w.box.erase(it);
                return MPI_SUCCESS;
            }
        }
        w.cv.wait(lk);
    }
}

int MPI_Get_count(const MPI_Status* status, MPI_Datatype type, int* count)
{
    *count = (int)(status->bytes / (long)type_of(type).extent);
    return MPI_SUCCESS;
}

int MPI_Type_create_struct(int count, const int* blocklens, const MPI_Aint* displs, const MPI_Datatype* types,
                           MPI_Datatype* newtype)
{
    TypeInfo ti{ {}, 0, 1, false };
    size_t end = 0;
    for (int k = 0; k < count; ++k) {
        const TypeInfo& m = type_of(types[k]);
        for (int b = 0; b < blocklens[k]; ++b)
            for (const Block& blk : m.blocks) ti.blocks.push_back(Block{ (size_t)displs[k] + b * m.extent + blk.off, blk.len });
        if ((size_t)displs[k] + blocklens[k] * m.extent > end) end = (size_t)displs[k] + blocklens[k] * m.extent;
        if (m.align > ti.align) ti.align = m.align;
    }
    ti.extent = (end + ti.align - 1) / ti.align * ti.align;
    World& w = world();
    std::lock_guard<std::mutex> lk(w.mu);
    w.types.push_back(ti);
    *newtype = (MPI_Datatype)(w.types.size() - 1);
    return MPI_SUCCESS;
}

int MPI_Type_commit(MPI_Datatype*) { return MPI_SUCCESS; }

} // extern "C"
