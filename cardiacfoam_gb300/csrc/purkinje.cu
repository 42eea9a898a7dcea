// Purkinje conduction network on the GPU: ConductionSystemDomain with the
// Monodomain1DSolver (src/electroModels/conductionSystemModels/
// monodomain1DSolver/monodomain1DSolver.C:36-190, src/electroModels/
// electroDomains/conductionSystemDomain/conductionSystemDomain.C,
// conductionGraph.H) and the reaction-diffusion PVJ coupling to a monodomain
// context (src/electroModels/electroCouplers/pvjCoupler/reactionDiffusion/
// reactionDiffusionPvjCoupler.C:36-164, pvjCoupler/pvjMapper.C).
//
// A network step is Strang split: the ionic model over dt/2 (the cfg_ionic
// kernels, tissue mode), the implicit cable step, the ionic model over the
// second dt/2.  The cable matrix of a tree is solved exactly by Hines
// elimination.  The reference eliminates node by node in reverse BFS order
// (children before parents) and substitutes in BFS order; here the tree is cut
// into BFS levels, so one block eliminates a whole level at once: every
// parent of the level subtracts its children's contributions in the order the
// reference visits them (reverse BFS), then the next level up; substitution
// runs level by level downwards.  Each accumulator sees the reference's
// operations in the reference's order, so the solution is bitwise the
// sequential one.  The matrix coefficients depend only on dt and the graph,
// and are assembled on the host (in the reference's order) when dt changes.
//
// Coupling: per terminal (PVJ) the tissue cell holding the junction (the
// nearest cell centre) and the cells whose centres lie within pvjRadius; the
// current (Vnet - Vtissue)/R_pvj enters the network as a negative applied
// current (bidirectional mode) and the tissue as the source I/sphereVolume
// on the cells of the sphere, added to the box stimulus in the reference's
// order.  The coupled step follows staggeredElectrophysicsAdvanceScheme:
// secondary coupling, the network's advance, primary coupling, the
// myocardium's advance.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "host_common.h"
#include "ionic_host.h"
#include "monodomain_host.h"

namespace {

constexpr int kPkBlock = 1024;

// rhs = Vm - dt Iion + dt Iapp / (chi Cm); Iapp from the root stimulus and
// the terminal currents (assembleAppliedCurrent); diag reset to its base
struct PkRhsArgs {
    long long n;
    double dt, chicm, t0;
    int root;
    double root_start, root_end, root_intensity;
    const int* term_off;    // [n+1] node -> its terminals (in terminal order)
    const int* term_idx;
    const double* term_current;
    const double* vm;
    const double* iion;
    const double* diag0;
    double* diag;
    double* rhs;
};

__global__ void k_pk_rhs(PkRhsArgs a)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    double app = 0.0;
    if (i == a.root && a.t0 >= a.root_start && a.t0 <= a.root_end) app += a.root_intensity;
    for (int k = a.term_off[i]; k < a.term_off[i + 1]; ++k) app -= a.term_current[a.term_idx[k]];
    a.rhs[i] = a.vm[i] - a.dt * a.iion[i] + a.dt * app / a.chicm;
    a.diag[i] = a.diag0[i];
}

struct HinesArgs {
    int n_levels;
    const int* level_off;   // [n_levels+1] ranges of `order` (BFS order = by level)
    const int* order;
    const int* parent;
    const int* child_off;   // [n+1] children of each node in reverse BFS order
    const int* children;
    const double* pc;       // row child -> column parent
    const double* cc;       // row parent -> column child
    double* diag;
    double* rhs;
    double* vm;
};

// One block: elimination from the deepest level up, then substitution down.
__global__ void __launch_bounds__(kPkBlock) k_pk_hines(HinesArgs a)
{
    for (int L = a.n_levels - 1; L >= 1; --L) {
        // parents on level L-1 take their children's contributions
        for (int k = a.level_off[L - 1] + threadIdx.x; k < a.level_off[L]; k += blockDim.x) {
            const int p = a.order[k];
            double d = a.diag[p], r = a.rhs[p];
            for (int j = a.child_off[p]; j < a.child_off[p + 1]; ++j) {
                const int c = a.children[j];
                const double factor = a.cc[c] / a.diag[c];
                d -= factor * a.pc[c];
                r -= factor * a.rhs[c];
            }
            a.diag[p] = d;
            a.rhs[p] = r;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const int root = a.order[0];
        a.vm[root] = a.rhs[root] / a.diag[root];
    }
    __syncthreads();
    for (int L = 1; L < a.n_levels; ++L) {
        for (int k = a.level_off[L] + threadIdx.x; k < a.level_off[L + 1]; k += blockDim.x) {
            const int c = a.order[k];
            a.vm[c] = (a.rhs[c] - a.pc[c] * a.vm[a.parent[c]]) / a.diag[c];
        }
        __syncthreads();
    }
}

// evaluateCoupling: I = (Vnet - Vtissue) / R_pvj per terminal and its
// volumetric source I / sphereVolume; the network's terminal current is I,
// or 0 (unidirectional, before the network's advance)
__global__ void k_pvj_eval(int n_term, const int* term_node, const int* term_cell,
                           const double* net_vm, const double* tissue_vm, double r_pvj,
                           const double* sphere_vol, int zero_network, double* term_current,
                           double* dep_value)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_term) return;
    const double I = (net_vm[term_node[i]] - tissue_vm[term_cell[i]]) / r_pvj;
    dep_value[i] = I / sphere_vol[i];
    term_current[i] = zero_network ? 0.0 : I;
}

}  // namespace

struct cfg_purkinje {
    cfg_ionic* ion = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    long long n = 0, n_edges = 0;
    double chi = 0, cm = 0, t = 0;
    int root = 0;
    double root_start = 1e300, root_duration = 0, root_intensity = 0;
    // graph, host
    std::vector<int> ea, eb, parent, order, rev, level_off, child_off, children, term_node,
        term_off, term_idx;
    std::vector<double> elen, econd, term_loc;
    // device
    int *d_level_off = nullptr, *d_order = nullptr, *d_parent = nullptr, *d_child_off = nullptr,
        *d_children = nullptr, *d_term_off = nullptr, *d_term_idx = nullptr,
        *d_term_node = nullptr;
    double *d_vm = nullptr, *d_iion = nullptr, *d_diag0 = nullptr, *d_pc = nullptr,
           *d_cc = nullptr, *d_diag = nullptr, *d_rhs = nullptr, *d_term_current = nullptr;
    double prepared_dt = 0.0;
    // coupling to a monodomain context
    cfg_monodomain* md = nullptr;
    int mode = 0;                  // 0 unidirectional, 1 bidirectional
    double r_pvj = 0, radius = 0;
    int* d_term_cell = nullptr;
    double *d_sphere_vol = nullptr, *d_dep_value = nullptr;
    int *d_dep_off = nullptr, *d_dep_term = nullptr;   // [cells+1] cell -> its terminals
    double* d_src_total = nullptr;
    std::vector<long long> h_term_cell;
    std::vector<double> h_sphere_vol;
};

using namespace cfg;

namespace {

void pk_free(cfg_purkinje* pk)
{
    if (pk->stream) cudaStreamSynchronize(pk->stream);
    for (int** p : {&pk->d_level_off, &pk->d_order, &pk->d_parent, &pk->d_child_off,
                    &pk->d_children, &pk->d_term_off, &pk->d_term_idx, &pk->d_term_node,
                    &pk->d_term_cell, &pk->d_dep_off, &pk->d_dep_term})
        dfree(*p);
    for (double** p : {&pk->d_vm, &pk->d_iion, &pk->d_diag0, &pk->d_pc, &pk->d_cc, &pk->d_diag,
                       &pk->d_rhs, &pk->d_term_current, &pk->d_sphere_vol, &pk->d_dep_value,
                       &pk->d_src_total})
        dfree(*p);
    if (pk->ion) cfg_ionic_destroy(pk->ion);
    if (pk->ev_in) cudaEventDestroy(pk->ev_in);
    if (pk->ev_out) cudaEventDestroy(pk->ev_out);
    if (pk->stream) cudaStreamDestroy(pk->stream);
    delete pk;
}

template <class T>
cudaError_t upload(T** dst, const std::vector<T>& v)
{
    cudaError_t e = dmalloc(dst, std::max<size_t>(v.size(), 1));
    if (!e && !v.empty()) e = cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    return e;
}

// Matrix coefficients of the cable step for dt (monodomain1DSolver.C:65-139):
// control lengths, diagonal 1 + sum of the incident coefficients, the
// parent/child off-diagonals, assembled in edge order as the reference does.
int prepare_dt(cfg_purkinje* pk, double dt)
{
    const size_t n = size_t(pk->n);
    const double chiCm = pk->chi * pk->cm;
    std::vector<double> diag(n, 1.0), pc(n, 0.0), cc(n, 0.0), clen(n, 0.0);
    for (size_t e = 0; e < size_t(pk->n_edges); ++e) {
        clen[size_t(pk->ea[e])] += 0.5 * pk->elen[e];
        clen[size_t(pk->eb[e])] += 0.5 * pk->elen[e];
    }
    for (size_t i = 0; i < n; ++i)
        if (clen[i] <= 1e-15)
            return fail(CFG_ERR_INVALID, "node %zu has zero 1D control length", i);
    for (size_t e = 0; e < size_t(pk->n_edges); ++e) {
        const int a = pk->ea[e], b = pk->eb[e];
        const double edgeCoeff = pk->econd[e] / pk->elen[e];
        const double coeffA = dt * edgeCoeff / (chiCm * clen[size_t(a)]);
        const double coeffB = dt * edgeCoeff / (chiCm * clen[size_t(b)]);
        diag[size_t(a)] += coeffA;
        diag[size_t(b)] += coeffB;
        if (pk->parent[size_t(a)] == b) {
            pc[size_t(a)] = -coeffA;
            cc[size_t(a)] = -coeffB;
        } else {
            pc[size_t(b)] = -coeffB;
            cc[size_t(b)] = -coeffA;
        }
    }
    CFG_CUDA_TRY(cudaMemcpyAsync(pk->d_diag0, diag.data(), n * sizeof(double),
                                 cudaMemcpyHostToDevice, pk->stream));
    CFG_CUDA_TRY(cudaMemcpyAsync(pk->d_pc, pc.data(), n * sizeof(double), cudaMemcpyHostToDevice,
                                 pk->stream));
    CFG_CUDA_TRY(cudaMemcpyAsync(pk->d_cc, cc.data(), n * sizeof(double), cudaMemcpyHostToDevice,
                                 pk->stream));
    CFG_CUDA_TRY(cudaStreamSynchronize(pk->stream));
    pk->prepared_dt = dt;
    return CFG_OK;
}

// Monodomain1DSolver::advance(t0, dt) on the network's stream.
int advance(cfg_purkinje* pk, double t0, double dt)
{
    if (dt != pk->prepared_dt)
        if (int rc = prepare_dt(pk, dt)) return rc;
    if (int rc = cfg_ionic_solve_device(pk->ion, t0, dt / 2.0, pk->d_vm, pk->d_iion)) return rc;
    PkRhsArgs r{};
    r.n = pk->n;
    r.dt = dt;
    r.chicm = pk->chi * pk->cm;
    r.t0 = t0;
    r.root = pk->root;
    r.root_start = pk->root_start;
    r.root_end = pk->root_start + pk->root_duration;
    r.root_intensity = pk->root_intensity;
    r.term_off = pk->d_term_off;
    r.term_idx = pk->d_term_idx;
    r.term_current = pk->d_term_current;
    r.vm = pk->d_vm;
    r.iion = pk->d_iion;
    r.diag0 = pk->d_diag0;
    r.diag = pk->d_diag;
    r.rhs = pk->d_rhs;
    k_pk_rhs<<<unsigned((pk->n + 255) / 256), 256, 0, pk->stream>>>(r);
    HinesArgs h{};
    h.n_levels = int(pk->level_off.size()) - 1;
    h.level_off = pk->d_level_off;
    h.order = pk->d_order;
    h.parent = pk->d_parent;
    h.child_off = pk->d_child_off;
    h.children = pk->d_children;
    h.pc = pk->d_pc;
    h.cc = pk->d_cc;
    h.diag = pk->d_diag;
    h.rhs = pk->d_rhs;
    h.vm = pk->d_vm;
    k_pk_hines<<<1, kPkBlock, 0, pk->stream>>>(h);
    CFG_CUDA_TRY(cudaGetLastError());
    return cfg_ionic_solve_device(pk->ion, t0 + (dt / 2.0), dt / 2.0, pk->d_vm, pk->d_iion);
}

}  // namespace

namespace cfg {

// The network part of a coupled monodomain step, enqueued before the
// myocardium's step: secondary coupling, the network's advance, primary
// coupling on the network's stream (after the context's earlier work), then
// the tissue's source (box stimulus plus the deposits) on the context's
// stream.
int purkinje_prepare_coupled_step(cfg_purkinje* pk, cfg_monodomain* md, double t0, double dt)
{
    const int nt = int(pk->term_node.size());
    CFG_CUDA_TRY(cudaEventRecord(pk->ev_in, md->stream));
    CFG_CUDA_TRY(cudaStreamWaitEvent(pk->stream, pk->ev_in, 0));
    const unsigned g = unsigned((nt + 127) / 128);
    if (nt)
        k_pvj_eval<<<g, 128, 0, pk->stream>>>(nt, pk->d_term_node, pk->d_term_cell, pk->d_vm,
                                              md->d_vm, pk->r_pvj, pk->d_sphere_vol,
                                              pk->mode == 0, pk->d_term_current, pk->d_dep_value);
    if (int rc = advance(pk, t0, dt)) return rc;
    if (nt)
        k_pvj_eval<<<g, 128, 0, pk->stream>>>(nt, pk->d_term_node, pk->d_term_cell, pk->d_vm,
                                              md->d_vm, pk->r_pvj, pk->d_sphere_vol, 0,
                                              pk->d_term_current, pk->d_dep_value);
    CFG_CUDA_TRY(cudaGetLastError());
    CFG_CUDA_TRY(cudaEventRecord(pk->ev_out, pk->stream));
    CFG_CUDA_TRY(cudaStreamWaitEvent(md->stream, pk->ev_out, 0));
    pk->t = t0 + dt;
    return monodomain_source_total(md, t0, pk->d_dep_off, pk->d_dep_term, pk->d_dep_value,
                                   pk->d_src_total);
}

int purkinje_check(cfg_purkinje* pk) { return ionic_check_status(pk->ion); }

void purkinje_detach(cfg_purkinje* pk)
{
    if (pk) pk->md = nullptr;
}

}  // namespace cfg

extern "C" {

int cfg_purkinje_create(const cfg_purkinje_desc* d, cfg_purkinje** out)
{
    clear_error();
    if (!d || !out) return fail(CFG_ERR_INVALID, "null argument");
    *out = nullptr;
    if (d->n_edges < 1 || !d->edge_a || !d->edge_b || !d->edge_length || !d->edge_conductance)
        return fail(CFG_ERR_INVALID, "the network needs conductionEdges");
    if (!(d->chi > 0) || !(d->cm > 0)) return fail(CFG_ERR_INVALID, "chi and cm must be positive");
    if (d->n_pvj < 0 || (d->n_pvj > 0 && (!d->pvj_nodes || !d->pvj_locations)))
        return fail(CFG_ERR_INVALID, "pvjNodes and pvjLocations must be given together");
    const long long ne = d->n_edges;
    int maxn = 0;
    for (long long e = 0; e < ne; ++e) {
        if (d->edge_a[e] < 0 || d->edge_b[e] < 0)
            return fail(CFG_ERR_INVALID, "edge %lld has a negative node", e);
        if (!(d->edge_length[e] > 0))
            return fail(CFG_ERR_INVALID, "edge %lld has a non-positive length", e);
        maxn = std::max(maxn, std::max(d->edge_a[e], d->edge_b[e]));
    }
    const long long n = (long long)maxn + 1;
    if (ne != n - 1)
        return fail(CFG_ERR_INVALID, "Conduction graph has %lld nodes but %lld edges. A tree "
                                     "requires exactly N-1 = %lld edges.", n, ne, n - 1);
    if (d->ionic.n_cells != n)
        return fail(CFG_ERR_INVALID, "the ionic model has %lld integration points, the network "
                                     "%lld nodes", d->ionic.n_cells, n);
    if (d->ionic.solve_vm_within_ode)
        return fail(CFG_ERR_INVALID, "the network step needs solveVmWithinODESolver false");
    if (d->root_node < 0 || d->root_node >= n)
        return fail(CFG_ERR_INVALID, "rootStimulus node %d is not in the network", d->root_node);
    for (int i = 0; i < d->n_pvj; ++i)
        if (d->pvj_nodes[i] < 0 || d->pvj_nodes[i] >= n)
            return fail(CFG_ERR_INVALID, "pvjNodes[%d]=%d is not in the network", i,
                        d->pvj_nodes[i]);
    cfg_purkinje* pk = new cfg_purkinje();
    auto bail = [&](int rc) { pk_free(pk); return rc; };
    pk->n = n;
    pk->n_edges = ne;
    pk->chi = d->chi;
    pk->cm = d->cm;
    pk->root = d->root_node;
    pk->root_start = d->root_start;
    pk->root_duration = d->root_duration;
    pk->root_intensity = d->root_intensity;
    pk->ea.assign(d->edge_a, d->edge_a + ne);
    pk->eb.assign(d->edge_b, d->edge_b + ne);
    pk->elen.assign(d->edge_length, d->edge_length + ne);
    pk->econd.assign(d->edge_conductance, d->edge_conductance + ne);
    // conductionGraph::buildTreeTopology: adjacency in edge order, BFS from 0
    std::vector<int> deg(size_t(n) + 1, 0), adj(size_t(2 * ne)), fill(size_t(n), 0);
    for (long long e = 0; e < ne; ++e) {
        deg[size_t(pk->ea[e]) + 1]++;
        deg[size_t(pk->eb[e]) + 1]++;
    }
    for (long long i = 0; i < n; ++i) deg[size_t(i) + 1] += deg[size_t(i)];
    for (long long e = 0; e < ne; ++e) {
        const int a = pk->ea[e], b = pk->eb[e];
        adj[size_t(deg[size_t(a)] + fill[size_t(a)]++)] = b;
        adj[size_t(deg[size_t(b)] + fill[size_t(b)]++)] = a;
    }
    pk->parent.assign(size_t(n), -1);
    pk->order.assign(size_t(n), 0);
    std::vector<int> depth(size_t(n), 0);
    std::vector<char> seen(size_t(n), 0);
    long long head = 0, tail = 0;
    pk->order[size_t(tail++)] = 0;
    seen[0] = 1;
    while (head < tail) {
        const int v = pk->order[size_t(head++)];
        for (int k = deg[size_t(v)]; k < deg[size_t(v) + 1]; ++k) {
            const int w = adj[size_t(k)];
            if (!seen[size_t(w)]) {
                seen[size_t(w)] = 1;
                pk->parent[size_t(w)] = v;
                depth[size_t(w)] = depth[size_t(v)] + 1;
                pk->order[size_t(tail++)] = w;
            }
        }
    }
    if (tail != n) {
        delete pk;
        return fail(CFG_ERR_INVALID, "Conduction graph is not connected: BFS from node 0 "
                                     "reached %lld of %lld nodes.", tail, n);
    }
    pk->rev.assign(pk->order.rbegin(), pk->order.rend());
    // BFS order is sorted by depth: the levels are its ranges
    pk->level_off.push_back(0);
    for (long long k = 1; k < n; ++k)
        if (depth[size_t(pk->order[size_t(k)])] != depth[size_t(pk->order[size_t(k - 1)])])
            pk->level_off.push_back(int(k));
    pk->level_off.push_back(int(n));
    // children of each node in reverse BFS order (the elimination's order)
    pk->child_off.assign(size_t(n) + 1, 0);
    for (long long k = 0; k < n; ++k) {
        const int p = pk->parent[size_t(pk->rev[size_t(k)])];
        if (p >= 0) pk->child_off[size_t(p) + 1]++;
    }
    for (long long i = 0; i < n; ++i) pk->child_off[size_t(i) + 1] += pk->child_off[size_t(i)];
    pk->children.assign(size_t(std::max<long long>(n - 1, 1)), 0);
    {
        std::vector<int> f(size_t(n), 0);
        for (long long k = 0; k < n; ++k) {
            const int c = pk->rev[size_t(k)], p = pk->parent[size_t(c)];
            if (p >= 0) pk->children[size_t(pk->child_off[size_t(p)] + f[size_t(p)]++)] = c;
        }
    }
    // terminals per node, in terminal order
    pk->term_node.assign(d->pvj_nodes, d->pvj_nodes + d->n_pvj);
    pk->term_loc.assign(d->pvj_locations, d->pvj_locations + 3 * d->n_pvj);
    pk->term_off.assign(size_t(n) + 1, 0);
    for (int i = 0; i < d->n_pvj; ++i) pk->term_off[size_t(pk->term_node[size_t(i)]) + 1]++;
    for (long long i = 0; i < n; ++i) pk->term_off[size_t(i) + 1] += pk->term_off[size_t(i)];
    pk->term_idx.assign(size_t(std::max(d->n_pvj, 1)), 0);
    {
        std::vector<int> f(size_t(n), 0);
        for (int i = 0; i < d->n_pvj; ++i) {
            const int v = pk->term_node[size_t(i)];
            pk->term_idx[size_t(pk->term_off[size_t(v)] + f[size_t(v)]++)] = i;
        }
    }
    cudaError_t e = cudaStreamCreateWithFlags(&pk->stream, cudaStreamNonBlocking);
    if (!e) e = cudaEventCreateWithFlags(&pk->ev_in, cudaEventDisableTiming);
    if (!e) e = cudaEventCreateWithFlags(&pk->ev_out, cudaEventDisableTiming);
    if (e) return bail(fail(CFG_ERR_CUDA, "stream: %s", cudaGetErrorString(e)));
    if (int rc = ionic_create(&d->ionic, pk->stream, &pk->ion)) return bail(rc);
    // ionicModel::vmRest (ionicModel.H:305-315): the model's state 0 in V
    double vm_rest = -0.084;
    {
        std::vector<double> C(size_t(std::max(pk->ion->ops->nc, 1)), 0.0),
            y(size_t(pk->ion->ops->ns), 0.0);
        pk->ion->ops->host_init(C.data(), y.data(), pk->ion->tissue, nullptr);
        const double u = y[0];
        switch (pk->ion->ops->vm_map) {
        case CFG_VM_ALIEV: vm_rest = (u * 100.0 - 80.0) * 1e-3; break;
        case CFG_VM_BUENO: vm_rest = (u * 85.7 - 84.0) * 1e-3; break;
        case CFG_VM_IDENTITY: vm_rest = u; break;
        default: vm_rest = u * 1e-3;
        }
    }
    std::vector<double> v0(size_t(n), vm_rest), zero(size_t(std::max(d->n_pvj, 1)), 0.0);
    if (!e) e = upload(&pk->d_level_off, pk->level_off);
    if (!e) e = upload(&pk->d_order, pk->order);
    if (!e) e = upload(&pk->d_parent, pk->parent);
    if (!e) e = upload(&pk->d_child_off, pk->child_off);
    if (!e) e = upload(&pk->d_children, pk->children);
    if (!e) e = upload(&pk->d_term_off, pk->term_off);
    if (!e) e = upload(&pk->d_term_idx, pk->term_idx);
    if (!e) e = upload(&pk->d_term_node, pk->term_node);
    if (!e) e = upload(&pk->d_vm, v0);
    if (!e) e = upload(&pk->d_term_current, zero);
    for (double** p : {&pk->d_iion, &pk->d_diag0, &pk->d_pc, &pk->d_cc, &pk->d_diag, &pk->d_rhs})
        if (!e) e = dmalloc(p, size_t(n));
    if (!e) e = cudaMemset(pk->d_iion, 0, size_t(n) * sizeof(double));
    if (e) return bail(fail(CFG_ERR_CUDA, "network allocation: %s", cudaGetErrorString(e)));
    *out = pk;
    return CFG_OK;
}

int cfg_purkinje_step(cfg_purkinje* pk, double dt)
{
    if (!pk) return fail(CFG_ERR_INVALID, "null network");
    if (!(dt > 0)) return fail(CFG_ERR_INVALID, "deltaT must be positive");
    if (pk->md)
        return fail(CFG_ERR_INVALID, "a coupled network advances with its monodomain context");
    if (int rc = advance(pk, pk->t, dt)) return rc;
    pk->t = pk->t + dt;
    CFG_CUDA_TRY(cudaStreamSynchronize(pk->stream));
    return ionic_check_status(pk->ion);
}

int cfg_purkinje_couple(cfg_purkinje* pk, cfg_monodomain* md, const cfg_mesh_desc* m,
                        double r_pvj, double pvj_radius, int bidirectional)
{
    if (!pk || !md || !m) return fail(CFG_ERR_INVALID, "null argument");
    if (pk->md) return fail(CFG_ERR_INVALID, "the network is already coupled");
    if (md->pk) return fail(CFG_ERR_INVALID, "the context already has a network");
    if (m->n_cells != md->n || !m->centres || !m->volumes)
        return fail(CFG_ERR_INVALID, "the mesh (centres, volumes) of the context is needed");
    if (!(r_pvj > 0) || !(pvj_radius > 0))
        return fail(CFG_ERR_INVALID, "rPvj and pvjRadius must be positive");
    const long long nc = m->n_cells;
    const int nt = int(pk->term_node.size());
    // PVJMapper: the cell holding each junction (the nearest centre, the first
    // on ties), the cells within pvjRadius and their volume
    std::vector<int> term_cell(size_t(std::max(nt, 1)), 0);
    std::vector<double> sphere(size_t(std::max(nt, 1)), 0.0);
    std::vector<std::vector<int>> per_cell_terms;
    std::vector<std::pair<long long, int>> pairs;
    for (int i = 0; i < nt; ++i) {
        const double* x = pk->term_loc.data() + 3 * i;
        long long best = -1;
        double bd = 1e300;
        for (long long c = 0; c < nc; ++c) {
            const double* C = m->centres + 3 * c;
            const double dd[3] = {C[0] - x[0], C[1] - x[1], C[2] - x[2]};
            const double dist = std::sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]);
            if (dist < bd) { bd = dist; best = c; }
        }
        if (pvj_radius < std::cbrt(m->volumes[best]))
            return fail(CFG_ERR_INVALID, "pvjRadius is smaller than the local myocardium cell "
                                         "size for PVJ terminal %d", i);
        term_cell[size_t(i)] = int(best);
        double vol = 0.0;
        const size_t first = pairs.size();
        for (long long c = 0; c < nc; ++c) {
            const double* C = m->centres + 3 * c;
            const double dd[3] = {C[0] - x[0], C[1] - x[1], C[2] - x[2]};
            if (std::sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]) <= pvj_radius) {
                pairs.push_back({c, i});
                vol += m->volumes[c];
            }
        }
        if (vol <= 1e-15) {
            pairs.resize(first);
            pairs.push_back({best, i});
            vol = m->volumes[best];
        }
        sphere[size_t(i)] = vol;
    }
    // cell -> its terminals in deposit order (terminal order)
    std::vector<int> dep_off(size_t(nc) + 1, 0), dep_term(std::max<size_t>(pairs.size(), 1), 0);
    for (const auto& pr : pairs) dep_off[size_t(pr.first) + 1]++;
    for (long long c = 0; c < nc; ++c) dep_off[size_t(c) + 1] += dep_off[size_t(c)];
    {
        std::vector<int> f(size_t(nc), 0);
        for (const auto& pr : pairs)
            dep_term[size_t(dep_off[size_t(pr.first)] + f[size_t(pr.first)]++)] = pr.second;
    }
    cudaError_t e = upload(&pk->d_term_cell, term_cell);
    if (!e) e = upload(&pk->d_sphere_vol, sphere);
    if (!e) e = upload(&pk->d_dep_off, dep_off);
    if (!e) e = upload(&pk->d_dep_term, dep_term);
    if (!e) e = dmalloc(&pk->d_dep_value, size_t(std::max(nt, 1)));
    if (!e) e = dmalloc(&pk->d_src_total, size_t(nc));
    if (e) return fail(CFG_ERR_CUDA, "coupling allocation: %s", cudaGetErrorString(e));
    pk->h_term_cell.assign(term_cell.begin(), term_cell.end());
    pk->h_sphere_vol = sphere;
    pk->r_pvj = r_pvj;
    pk->radius = pvj_radius;
    pk->mode = bidirectional ? 1 : 0;
    pk->md = md;
    pk->t = md->t_host;
    return monodomain_attach_network(md, pk, pk->d_src_total);
}

int cfg_purkinje_get_field(cfg_purkinje* pk, int field, double* host)
{
    if (!pk || !host) return fail(CFG_ERR_INVALID, "null argument");
    const double* src = field == CFG_FIELD_VM ? pk->d_vm : field == CFG_FIELD_IION ? pk->d_iion
                                                                                  : nullptr;
    if (!src) return fail(CFG_ERR_INVALID, "field %d: the network has Vm and Iion", field);
    CFG_CUDA_TRY(cudaStreamSynchronize(pk->stream));
    CFG_CUDA_TRY(cudaMemcpy(host, src, size_t(pk->n) * sizeof(double), cudaMemcpyDeviceToHost));
    return CFG_OK;
}

int cfg_purkinje_terminal_current(cfg_purkinje* pk, double* host)
{
    if (!pk || !host) return fail(CFG_ERR_INVALID, "null argument");
    CFG_CUDA_TRY(cudaStreamSynchronize(pk->stream));
    if (!pk->term_node.empty())
        CFG_CUDA_TRY(cudaMemcpy(host, pk->d_term_current, pk->term_node.size() * sizeof(double),
                                cudaMemcpyDeviceToHost));
    return CFG_OK;
}

long long cfg_purkinje_nodes(const cfg_purkinje* pk) { return pk ? pk->n : 0; }
double cfg_purkinje_time(const cfg_purkinje* pk) { return pk ? pk->t : 0.0; }

int cfg_purkinje_destroy(cfg_purkinje* pk)
{
    if (!pk) return CFG_OK;
    if (pk->md) monodomain_attach_network(pk->md, nullptr, nullptr);
    pk_free(pk);
    return CFG_OK;
}

}  // extern "C"
