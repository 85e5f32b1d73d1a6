// ref_buffer_wrap.cc -- TEST INFRASTRUCTURE ONLY: a C interface to the reference's own immigrant
// buffer classes (src/buffer_manage.cc, include/buffer_manage.h), compiled in place from the
// reference's sources into oracle/_ref/libref_buffer.so with `real = float` (the
// ref_shim/config_f32.h force-include), so that the tests can feed them the same immigrant
// messages as the oracle's archipelago restatement and compare the buffers they hold.
//
// The classes keep their state in protected members; the Open* wrappers below expose it for
// reading (and ref_buf_assign replaces a FIFO-family buffer's members). Policies: 0 OnlineCluster, 1 BestSelect, 2 RandomSelect, 3 FIFO, 4 LIFO (the
// library's numbering). LIFO::SelectFromBuffer erases end() (undefined behaviour,
// buffer_manage.cc:309) and RandomSelect::SelectFromBuffer draws from rand(): ref_buf_select
// refuses both.
#include "buffer_manage.h"

namespace {

template <class B>
struct Open : B {
    explicit Open(int cap) : B(cap) {}
    Population &buffer() { return this->recv_buffer_; }
};

struct OpenCluster : OnlineCluster {
    explicit OpenCluster(int cap) : OnlineCluster(cap) {}
    Population &buffer() { return recv_buffer_; }
    Population &centres() { return cluster_centre_; }
    vector<int> &members() { return cluster_member_num_; }
    vector<int> &flags() { return flag_updated_; }
};

struct Handle {
    int policy;
    BufferManage *b;
};

Population &buffer_of(Handle *h)
{
    switch (h->policy) {
    case 0: return static_cast<OpenCluster *>(h->b)->buffer();
    case 1: return static_cast<Open<BestSelect> *>(h->b)->buffer();
    case 2: return static_cast<Open<RandomSelect> *>(h->b)->buffer();
    case 3: return static_cast<Open<FIFO> *>(h->b)->buffer();
    default: return static_cast<Open<LIFO> *>(h->b)->buffer();
    }
}

void to_rows(const Population &p, int dim, float *X, float *fit)
{
    for (size_t i = 0; i < p.size(); ++i) {
        for (int j = 0; j < dim; ++j) X[i * (size_t)dim + j] = p[i].elements[j];
        fit[i] = p[i].fitness_value;
    }
}

}  // namespace

extern "C" {

void *ref_buf_create(int policy, int capacity)
{
    Handle *h = new Handle{policy, nullptr};
    switch (policy) {
    case 0: h->b = new OpenCluster(capacity); break;
    case 1: h->b = new Open<BestSelect>(capacity); break;
    case 2: h->b = new Open<RandomSelect>(capacity); break;
    case 3: h->b = new Open<FIFO>(capacity); break;
    case 4: h->b = new Open<LIFO>(capacity); break;
    default: delete h; return nullptr;
    }
    return h;
}

void ref_buf_destroy(void *p)
{
    Handle *h = static_cast<Handle *>(p);
    delete h->b;
    delete h;
}

// One received message (UpdateBuffer, as CheckAndRecvEmigrations calls it, src/migrate.cc:71-103):
// n individuals of dim elements (rows of X) with their fitness.
int ref_buf_update(void *p, int n, int dim, const float *X, const float *fit)
{
    Handle *h = static_cast<Handle *>(p);
    Population msg((size_t)n);
    for (int i = 0; i < n; ++i) {
        msg[i].elements.assign(X + (size_t)i * dim, X + (size_t)(i + 1) * dim);
        msg[i].fitness_value = fit[i];
    }
    return h->b->UpdateBuffer(msg);
}

// SelectFromBuffer(emigration_export, k) into X_out / fit_out (room for the buffer's size);
// returns the number selected, or -1 for the policies that cannot be replayed here.
int ref_buf_select(void *p, int k, int dim, float *X_out, float *fit_out)
{
    Handle *h = static_cast<Handle *>(p);
    if (h->policy == 2 || h->policy == 4) return -1;
    Population out;
    h->b->SelectFromBuffer(out, k);
    to_rows(out, dim, X_out, fit_out);
    return (int)out.size();
}

// Replaces the buffer's members with n given individuals (FIFO-family policies only): lets a test
// carry on comparing UpdateBuffer after a selection it cannot replay (RandomSelect, LIFO).
int ref_buf_assign(void *p, int n, int dim, const float *X, const float *fit)
{
    Handle *h = static_cast<Handle *>(p);
    if (h->policy == 0) return -1;
    Population &b = buffer_of(h);
    b.assign((size_t)n, Individual());
    for (int i = 0; i < n; ++i) {
        b[i].elements.assign(X + (size_t)i * dim, X + (size_t)(i + 1) * dim);
        b[i].fitness_value = fit[i];
    }
    return 0;
}

int ref_buf_size(void *p) { return (int)buffer_of(static_cast<Handle *>(p)).size(); }

// The buffer's members in vector order.
void ref_buf_entries(void *p, int dim, float *X, float *fit) { to_rows(buffer_of(static_cast<Handle *>(p)), dim, X, fit); }

// OnlineCluster only: centres (size x dim), member counts and update flags.
int ref_buf_clusters(void *p, int dim, float *centres, int *members, int *flags)
{
    Handle *h = static_cast<Handle *>(p);
    if (h->policy != 0) return -1;
    OpenCluster *c = static_cast<OpenCluster *>(h->b);
    for (size_t i = 0; i < c->centres().size(); ++i) {
        for (int j = 0; j < dim; ++j) centres[i * (size_t)dim + j] = c->centres()[i].elements[j];
        members[i] = c->members()[i];
        flags[i] = c->flags()[i];
    }
    return (int)c->centres().size();
}

}  // extern "C"
