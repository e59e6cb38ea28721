// batch.cu -- many tournaments per launch: one work list per tree-level step.
//
// A forest holds T independent tournaments of uneven size, each with its own
// tree geometry (plan_geometry) and tree buffers, all in one arena.  For a
// chunk of quadrature nodes every step of the single-plan sequence -- leaf
// blocks, the products of tree level l, the spectral transitions, the
// propagate of level l, the per-player divide -- becomes ONE launch that
// covers every tournament having that step: a work list of descriptors (the
// kernel's argument block for one tournament level) plus a table that maps
// each CTA of the launch to (descriptor, block).  Kernels whose shared memory
// depends on a transform size are split into one list per size.  Players of
// all tournaments share the node-major arrays a[q][N] and contrib[q][N], so
// one accumulate and one scatter serve the whole forest.  The launch
// sequence of a run is captured once as a CUDA graph and replayed while the
// node count stays the same.
//
// Every tournament's arithmetic is the single-plan path's, kernel for kernel,
// so batched equities equal single-plan equities bit for bit.  Tournaments
// whose levels need the multi-pass transforms (products beyond one CTA's
// shared memory) are solved by single plans after the forest.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <thread>

#include "batch.h"
#include "kernels.h"

namespace icmg {

static double now_ns() {
    return (double)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}
static size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }
static int ilog2l(long v) {
    int l = 0;
    while ((1L << l) < v) ++l;
    return l;
}

// run fn(i) for i in [0, count) on up to hardware_concurrency threads
template <class F>
static void parallel_for(int count, F fn) {
    int nt = (int)std::max(1u, std::thread::hardware_concurrency());
    nt = std::min(nt, std::max(1, count / 8));
    if (nt <= 1) {
        for (int i = 0; i < count; ++i) fn(i);
        return;
    }
    std::vector<std::thread> th;
    for (int w = 0; w < nt; ++w)
        th.emplace_back([&, w] {
            SortThreadCap cap(1);   // the members' sorts: one thread each
            for (int i = w; i < count; i += nt) fn(i);
        });
    for (auto &t : th) t.join();
}

// every level of the tree runs on one-CTA kernels
static bool fits_worklist(const Plan *p) {
    if (p->small || p->linear) return true;
    for (int l = 1; l < p->L; ++l) {
        const Level &v = p->lv[l], &c = p->lv[l - 1];
        if (v.kind == 1 && v.npairs > 0 && !fused_ok(v.fftn)) return false;
        if (v.kind == 2 && (c.deg > kSpecMaxD || v.deg / 2 > kSpecMaxD)) return false;
    }
    return true;
}

// ------------------------------------------------------------ step lists
namespace {
struct PhaseBuilder {
    std::vector<WStep> steps;
    // set before add() for packed steps: items of the descriptor, items per CTA
    int pack_items = 0, pack_cb = 1;
    template <class A>
    void add(WOp op, int key, const char *name, const A &a, size_t smem, double fq, int one = 0, int mem = -1,
             long span = 0, int nreal = 0, double fq0 = 0.0) {
        if (a.nbx <= 0) return;
        WStep *s = nullptr;
        for (auto &x : steps)
            if (x.op == op && x.key == key && x.one == one) s = &x;
        if (!s) {
            steps.emplace_back();
            s = &steps.back();
            s->op = op;
            s->key = key;
            s->one = one;
            s->name = name;
            s->esz = sizeof(A);
            s->packed = pack_items > 0 ? 1 : 0;
            s->cb = pack_cb;
        }
        const unsigned char *b = (const unsigned char *)&a;
        s->desc.insert(s->desc.end(), b, b + sizeof(A));
        if (s->packed)
            for (int j = 0; j < pack_items; ++j) s->tab.push_back(make_int2(s->nd, j));
        else
            for (int bx = 0; bx < a.nbx; ++bx) s->tab.push_back(make_int2(s->nd, bx));
        ++s->nd;
        s->smem = std::max(s->smem, smem);
        s->fq += fq;
        s->dmem.push_back(mem);
        s->dspan.push_back(span);
        s->dnreal.push_back(nreal);
        s->dfq.push_back(fq);
        s->dfq0.push_back(fq0);
    }
};
}  // namespace

static const int *zpre(const Plan *p) { return p->zskip ? p->d_z : nullptr; }

// descriptors of every step for Q nodes (pointers into the forest arena)
static void build_steps(Forest *f) {
    const int T = (int)f->tr.size();
    int Lmax = 0;
    for (Plan *p : f->tr) Lmax = std::max(Lmax, p->L);
    const double2 *tw = f->tw;
    const int logTW = f->logTW;
    const size_t aq = (size_t)f->Ntot;
    std::vector<PhaseBuilder> pre(1);
    std::deque<PhaseBuilder> ph;   // stable references while phases are added
    auto phase = [&]() -> PhaseBuilder & { ph.emplace_back(); return ph.back(); };

    std::vector<SubArgs> subs(T);
    std::vector<SubFlops> subfl(T);
    {   // leaf blocks (with the bottom schoolbook levels where they are fused)
        PhaseBuilder &b = phase();
        for (int t = 0; t < T; ++t) {
            Plan *p = f->tr[t];
            double fq = 0;
            if (p->small) {   // the whole pipeline in one CTA per node
                const SmallArgs A = small_args(p, p->d_S, p->d_node, p->d_payout, f->d_contrib + f->off[t], aq,
                                               nullptr);
                b.add(WOp::Small, p->B, "wl_small", A, A.smem, small_flops(p));
                continue;
            }
            if (p->linear) {   // one warp per node
                const LinearArgs A = linear_args(p, p->d_S, p->d_node, p->d_payout, f->d_a + f->off[t],
                                                 f->d_contrib + f->off[t], aq, nullptr, p->d_ck, zpre(p));
                b.add(WOp::Linear, A.R, "wl_linear", A, 0, linear_flops(p));
                continue;
            }
            if (p->Lf >= 1) {
                subs[t] = sub_args(p, p->Lf, p->d_S, p->d_node, f->d_a + f->off[t], aq, nullptr,
                                   f->d_contrib + f->off[t], false, true, &subfl[t]);
                // the levels' share is pruned like level Lf (profiler only)
                double lvl = 0.0;
                for (int l = 1; l <= p->Lf; ++l) lvl += subfl[t].build[l];
                b.add(WOp::SubBuild, p->B, "wl_sub_build", subs[t], sub_build_smem(p->B), lvl, 0, t, p->lv[p->Lf].deg,
                      p->lv[p->Lf].nreal, subfl[t].leaf);
                continue;
            }
            LeafArgs A = leaf_args(p->B, p->n, p->nblocks, p->d_S, p->d_node, f->d_a + f->off[t], aq, p->d_blockP,
                                   p->lv[0].P, p->lv[0].pst, p->lv[0].plen, &fq);
            b.add(WOp::Leaf, p->B, "wl_leaf", A, 0, fq);
        }
        PhaseBuilder &c = phase();
        for (int t = 0; t < T; ++t) {
            Plan *p = f->tr[t];
            if (!p->small && !p->linear && p->L >= 2 && p->lv[1].kind == 2) {
                double fq = 0;
                size_t sm = 0;
                SpecInitArgs A = spec_init_args(p->lv[0], tw, logTW, &fq, &sm);
                A.z.zp = zpre(p);
                c.add(WOp::SpecInit, A.logd, "wl_spec_init", A, sm, fq, 0, t, p->lv[0].deg, p->lv[0].nreal);
            }
        }
    }
    // products, level by level
    for (int l = 1; l < Lmax; ++l) {
        PhaseBuilder &b = phase();
        for (int t = 0; t < T; ++t) {
            Plan *p = f->tr[t];
            if (p->small || p->linear) continue;
            Level *lv = p->lv;
            double fq = 0;
            size_t sm = 0;
            if (l <= p->Lf) continue;   // in the subtree kernel
            if (l <= p->L - 2) {
                if (lv[l].kind == 2) {
                    SpecBuildArgs A = spec_build_args(lv[l - 1], lv[l], lv[l + 1].kind != 2, tw, logTW, &fq, &sm);
                    A.z.zp = zpre(p);
                    b.pack_items = lv[l].nreal;   // items of different members share CTAs
                    b.pack_cb = A.cb;   // items per CTA of the spectral work lists
                    b.add(WOp::SpecBuild, 2 * A.logD + (A.pspec ? 1 : 0), "wl_spec_build", A, sm, fq, 0, t, lv[l].deg,
                          lv[l].nreal);
                    b.pack_items = 0;
                } else if (lv[l].fft) {
                    if (lv[l].npairs > 0) {
                        FusedBuildArgs A = fused_build_args(lv[l - 1], lv[l], false, tw, logTW, &fq, &sm);
                        A.z.zp = zpre(p);
                        b.pack_items = lv[l].npairs;
                        b.pack_cb = A.cb;   // items per CTA of the fused kernels
                        b.add(WOp::FusedBuild, 2 * A.logN, "wl_fused_build", A, sm, fq, 0, t, lv[l].deg, lv[l].nreal);
                        b.pack_items = 0;
                    }
                    if (lv[l - 1].nreal & 1) {
                        SchoolBuildArgs A = school_build_args(lv[l - 1], lv[l], lv[l].npairs, &fq);
                        A.z.zp = zpre(p);
                        b.add(WOp::SchoolBuild, 0, "wl_school_build", A, 0, fq, 0, t, lv[l].deg, lv[l].nreal);
                    }
                } else {
                    SchoolBuildArgs A = school_build_args(lv[l - 1], lv[l], 0, &fq);
                    A.z.zp = zpre(p);
                    b.add(WOp::SchoolBuild, 0, "wl_school_build", A, 0, fq, 0, t, lv[l].deg, lv[l].nreal);
                }
            } else if (l == p->L - 1 && lv[l].fft && lv[l].npairs > 0) {
                // the root: child spectra for its propagate only
                FusedBuildArgs A = fused_build_args(lv[l - 1], lv[l], true, tw, logTW, &fq, &sm);
                b.pack_items = lv[l].npairs;
                b.pack_cb = A.cb;   // items per CTA of the fused kernels
                b.add(WOp::FusedBuild, 2 * A.logN + 1, "wl_fused_spectra", A, sm, fq);
                b.pack_items = 0;
            }
        }
        PhaseBuilder &c = phase();
        for (int t = 0; t < T; ++t) {
            Plan *p = f->tr[t];
            if (p->small || p->linear) continue;
            Level *lv = p->lv;
            if (l <= p->L - 2 && lv[l].kind != 2 && lv[l + 1].kind == 2) {
                double fq = 0;
                size_t sm = 0;
                SpecInitArgs A = spec_init_args(lv[l], tw, logTW, &fq, &sm);
                A.z.zp = zpre(p);
                c.add(WOp::SpecInit, A.logd, "wl_spec_init", A, sm, fq, 0, t, lv[l].deg, lv[l].nreal);
            }
        }
    }
    // propagate, root to leaves
    for (int l = Lmax - 1; l >= 1; --l) {
        PhaseBuilder &a = phase();
        for (int t = 0; t < T; ++t) {
            Plan *p = f->tr[t];
            if (p->small || p->linear) continue;
            Level *lv = p->lv;
            if (l > p->L - 1 || lv[l].kind != 2) continue;
            const bool root = (l == p->L - 1);
            double fq = 0;
            size_t sm = 0;
            if (root) {   // the payout's spectrum, shared by the nodes: once per run
                GspecArgs A = gspec_args(p->d_payout, 0, 0, p->k, lv[l].nreal, lv[l], lv[l].G, 0, nullptr, tw, logTW,
                                         &fq, &sm);
                pre[0].add(WOp::Gspec, A.logd, "wl_gspec_root", A, sm, fq, 1);
            } else if (lv[l + 1].kind != 2) {
                GspecArgs A = gspec_args(lv[l].g, lv[l].g_q, lv[l].gst, lv[l].glen, lv[l].nreal, lv[l], lv[l].G,
                                         lv[l].G_q, nullptr, tw, logTW, &fq, &sm);
                A.z.zp = zpre(p);
                a.add(WOp::Gspec, A.logd, "wl_gspec_init", A, sm, fq, 0, t, lv[l].deg, lv[l].nreal);
            }
        }
        PhaseBuilder &b = phase();
        for (int t = 0; t < T; ++t) {
            Plan *p = f->tr[t];
            if (p->small || p->linear) continue;
            Level *lv = p->lv;
            if (l > p->L - 1 || l <= p->Lf) continue;
            const bool root = (l == p->L - 1);
            const double *gp = root ? p->d_payout : lv[l].g;
            const size_t gp_q = root ? 0 : lv[l].g_q;
            const int gst_p = root ? 0 : lv[l].gst;
            const int gpl = root ? p->k : lv[l].glen;
            double fq = 0;
            size_t sm = 0;
            if (lv[l].kind == 2) {
                SpecPropArgs A = spec_prop_args(lv[l].G, root ? 0 : lv[l].G_q, lv[l - 1], lv[l],
                                                l - 1 >= 1 && lv[l - 1].kind == 2, nullptr, tw, logTW, &fq, &sm);
                A.z.zp = zpre(p);
                b.pack_items = lv[l].nreal;
                b.pack_cb = A.cb;   // items per CTA of the spectral work lists
                b.add(WOp::SpecProp, 2 * A.logD + (A.Gout ? 1 : 0), "wl_spec_prop", A, sm, fq, 0, t,
                      root ? 0 : lv[l].deg, lv[l].nreal);
                b.pack_items = 0;
            } else if (lv[l].fft) {
                if (lv[l].npairs > 0) {
                    FusedPropArgs A = fused_prop_args(gp, gp_q, gst_p, gpl, lv[l - 1], lv[l], nullptr, tw, logTW, &fq,
                                                      &sm);
                    A.z.zp = zpre(p);
                    b.pack_items = lv[l].npairs;
                    b.pack_cb = A.cb;   // items per CTA of the fused kernels
                    b.add(WOp::FusedProp, A.logN, "wl_fused_prop", A, sm, fq, 0, t, root ? 0 : lv[l].deg, lv[l].nreal);
                    b.pack_items = 0;
                }
                if (lv[l - 1].nreal & 1) {
                    SchoolPropArgs A = school_prop_args(gp, gp_q, gst_p, gpl, lv[l - 1], nullptr, 2 * lv[l].npairs, &fq);
                    A.z.zp = zpre(p);
                    b.add(WOp::SchoolProp, 0, "wl_school_prop", A, 0, fq, 0, t, lv[l - 1].deg, lv[l - 1].nreal);
                }
            } else {
                SchoolPropArgs A = school_prop_args(gp, gp_q, gst_p, gpl, lv[l - 1], nullptr, 0, &fq);
                A.z.zp = zpre(p);
                b.add(WOp::SchoolProp, 0, "wl_school_prop", A, 0, fq, 0, t, lv[l - 1].deg, lv[l - 1].nreal);
            }
        }
    }
    if (f->vjp) {   // adjoint passes: leaf blocks, up the tree, down the tree, players
        const size_t pq = (size_t)f->qc * f->Ntot;
        double *pA = f->node_terms ? f->d_part : nullptr, *pB = f->node_terms ? f->d_part + pq : nullptr;
        PhaseBuilder &u = phase();
        for (int t = 0; t < T; ++t)
            u.add(WOp::AdjLeafUp, f->tr[t]->B, "wl_adj_leaf_up", adj_leaf_up_args(f->tr[t], f->vb[t]), 0, 0.0);
        for (int l = 1; l < Lmax; ++l) {
            // spectral levels over coefficient children: the children's gbar as spectra first
            PhaseBuilder &cv = phase();
            for (int t = 0; t < T; ++t) {
                Plan *p = f->tr[t];
                if (l > p->L - 1 || p->lv[l].kind != 2 || p->lv[l - 1].kind == 2) continue;
                size_t sm = 0;
                const VspRealArgs R = vsp_gbar_real_args(p, f->vb[t], l, 0, tw, logTW, &sm);
                cv.add(WOp::AdjSpecReal, R.logM, "wl_adj_spec_real", R, sm, 0.0);
            }
            PhaseBuilder &b = phase();
            for (int t = 0; t < T; ++t) {
                Plan *p = f->tr[t];
                if (l > p->L - 1) continue;
                if (p->lv[l].kind == 2) {   // spectral level: the adjoint in the frequency domain
                    size_t sm = 0;
                    const VspUpArgs A = vsp_up_args(p, f->vb[t], l, 0, tw, logTW, &sm);
                    b.add(WOp::AdjSpecUp, A.logD, "wl_adj_spec_up", A, sm, 0.0);
                    continue;
                }
                AdjUpFusedArgs F;
                AdjUpSchoolArgs Sa;
                adj_up_args(p, f->vb[t], l, tw, logTW, F, Sa);
                b.pack_items = F.npairs;   // pairs of different members share CTAs
                b.pack_cb = F.nbx > 0 ? adj_items_per_cta(F.logN) : 1;
                b.add(WOp::AdjUpFused, F.logN, "wl_adj_up_fused", F, adj_up_smem(F.logN), 0.0);
                b.pack_items = 0;
                b.add(WOp::AdjUpSchool, 0, "wl_adj_up_school", Sa, 0, 0.0);
            }
        }
        for (int l = Lmax - 1; l >= 1; --l) {
            // spectral levels under a coefficient level: the parents' Pbar as folded spectra first
            PhaseBuilder &cv = phase();
            for (int t = 0; t < T; ++t) {
                Plan *p = f->tr[t];
                if (l >= p->L - 1 || p->lv[l].kind != 2 || p->lv[l + 1].kind == 2) continue;
                size_t sm = 0;
                const VspRealArgs R = vsp_pbar_real_args(p, f->vb[t], l, 0, tw, logTW, &sm);
                cv.add(WOp::AdjSpecReal, R.logM, "wl_adj_spec_real", R, sm, 0.0);
            }
            PhaseBuilder &b = phase();
            for (int t = 0; t < T; ++t) {
                Plan *p = f->tr[t];
                if (l > p->L - 1) continue;
                if (p->lv[l].kind == 2) {
                    size_t sm = 0;
                    const VspDownArgs A = vsp_down_args(p, f->vb[t], l, 0, tw, logTW, &sm);
                    b.add(WOp::AdjSpecDown, 2 * A.logD + (A.PFout ? 1 : 0), "wl_adj_spec_down", A, sm, 0.0);
                    continue;
                }
                AdjDownFusedArgs F;
                AdjDownSchoolArgs Sa;
                adj_down_args(p, f->vb[t], l, tw, logTW, F, Sa);
                b.pack_items = F.npairs;
                b.pack_cb = F.nbx > 0 ? adj_items_per_cta(F.logN) : 1;
                b.add(WOp::AdjDownFused, F.logN, "wl_adj_down_fused", F, adj_down_smem(F.logN), 0.0);
                b.pack_items = 0;
                b.add(WOp::AdjDownSchool, 0, "wl_adj_down_school", Sa, 0, 0.0);
            }
        }
        PhaseBuilder &d = phase();
        for (int t = 0; t < T; ++t) {
            Plan *p = f->tr[t];
            const AdjLeafDownArgs A =
                adj_leaf_down_args(p, f->vb[t], pA ? pA + f->off[t] : nullptr, pB ? pB + f->off[t] : nullptr);
            d.add(WOp::AdjLeafDown, p->B, "wl_adj_leaf_down", A, 0, 0.0);
        }
    } else {   // per-player divide
        PhaseBuilder &b = phase();
        for (int t = 0; t < T; ++t) {
            Plan *p = f->tr[t];
            const int L = p->L;
            if (p->small || p->linear) continue;
            if (p->Lf >= 1) {   // the bottom levels' propagate and the division
                double lvl = 0.0;
                for (int l = 1; l <= p->Lf; ++l) lvl += subfl[t].prop[l];
                b.add(WOp::SubProp, p->B, "wl_sub_prop", subs[t], sub_prop_smem(p->B), lvl, 0, t, p->lv[0].deg,
                      p->lv[0].nreal, subfl[t].divide);
                continue;
            }
            const double *g0 = (L == 1) ? p->d_payout : p->lv[0].g;
            const size_t g0_q = (L == 1) ? 0 : p->lv[0].g_q;
            const int gst0 = (L == 1) ? 0 : p->lv[0].gst;
            double fq = 0;
            DivideArgs A = divide_args(p->B, p->n, p->k, p->nblocks, p->d_S, p->d_node, f->d_a + f->off[t], aq,
                                       p->d_blockP, g0, g0_q, gst0, nullptr, f->d_contrib + f->off[t], &fq);
            b.add(WOp::Divide, p->B, "wl_divide", A, 0, fq, 0, t, 1, p->n);
        }
    }
    f->pre = std::move(pre[0].steps);
    f->steps.clear();
    for (auto &b : ph)
        for (auto &s : b.steps) f->steps.push_back(std::move(s));
}

// descriptors and tables into one device buffer
static int upload_steps(Forest *f, std::string &err) {
    size_t bytes = 0;
    auto size_of = [&](std::vector<WStep> &v) {
        for (auto &s : v) bytes += align256(s.desc.size()) + align256(s.tab.size() * sizeof(int2));
    };
    size_of(f->pre);
    size_of(f->steps);
    if (bytes > f->desc_cap) {
        if (f->d_desc) cudaFree(f->d_desc);
        f->d_desc = nullptr;
        f->desc_cap = 0;
        cudaError_t e = dev_alloc((void **)&f->d_desc, bytes, f->stream, false);
        if (e != cudaSuccess) { err = std::string("work lists: ") + cudaGetErrorString(e); return -1; }
        f->desc_cap = bytes;
    }
    std::vector<unsigned char> h(bytes, 0);
    size_t off = 0;
    auto place = [&](std::vector<WStep> &v) {
        for (auto &s : v) {
            memcpy(h.data() + off, s.desc.data(), s.desc.size());
            s.d_desc = f->d_desc + off;
            off += align256(s.desc.size());
            memcpy(h.data() + off, s.tab.data(), s.tab.size() * sizeof(int2));
            s.d_tab = (const int2 *)(f->d_desc + off);
            off += align256(s.tab.size() * sizeof(int2));
        }
    };
    place(f->pre);
    place(f->steps);
    cudaError_t e = cudaMemcpyAsync(f->d_desc, h.data(), bytes, cudaMemcpyHostToDevice, f->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(f->stream);
    if (e != cudaSuccess) { err = std::string("work list upload: ") + cudaGetErrorString(e); return -1; }
    return 0;
}

// flops of one launch over nq nodes, without the pruned (node, q) pairs
static double step_flops(const Forest *f, const WStep &s, int nq, int q0) {
    if (s.one) return s.fq;
    double fl = 0.0;
    for (int d = 0; d < s.nd; ++d) {
        const int m = s.dmem[d];
        const long span = s.dspan[d];
        const int nr = s.dnreal[d];
        if (m < 0 || span <= 0 || nr <= 0 || f->h_z.empty() || !f->tr[m]->zskip) {
            fl += (s.dfq[d] + s.dfq0[d]) * nq;
            continue;
        }
        const int *z = f->h_z.data() + (size_t)m * f->Q;
        double hot = 0.0;
        for (int q = 0; q < nq; ++q) hot += nr - std::min<long>(nr, z[q0 + q] / span);
        fl += s.dfq[d] * hot / nr + s.dfq0[d] * nq;
    }
    return fl;
}

static void launch_step(Forest *f, const WStep &s, int nq, int q0) {
    const int nctas = (int)s.tab.size();
    const int qn = s.one ? 1 : nq;
    if (f->prof.on) f->prof.begin(s.name, step_flops(f, s, qn, q0), f->stream);
    if (s.packed) {
        if (s.op == WOp::FusedBuild || s.op == WOp::FusedProp)
            launch_packed_fused(s.op, s.d_desc, s.d_tab, nctas, s.cb, qn, q0, s.smem, f->stream);
        else if (s.op == WOp::AdjUpFused || s.op == WOp::AdjDownFused)
            launch_packed_adj(s.op, s.d_desc, s.d_tab, nctas, s.cb, qn, q0, s.smem, f->stream);
        else
            launch_packed_spec(s.op, s.d_desc, s.d_tab, nctas, s.cb, qn, q0, s.smem, f->stream);
        f->prof.end(f->stream);
        ++f->launches;
        return;
    }
    switch (s.op) {
        case WOp::Leaf:
        case WOp::Divide:
        case WOp::SchoolBuild:
        case WOp::SchoolProp: launch_worklist_basic(s.op, s.key, s.d_desc, s.d_tab, nctas, qn, q0, f->stream); break;
        case WOp::SubBuild:
        case WOp::SubProp: launch_worklist_sub(s.op, s.key, s.d_desc, s.d_tab, nctas, qn, q0, s.smem, f->stream); break;
        case WOp::Small: launch_worklist_small(s.key, s.d_desc, s.d_tab, nctas, qn, q0, s.smem, f->stream); break;
        case WOp::Linear: launch_worklist_linear(s.key, s.d_desc, s.d_tab, nctas, qn, q0, f->stream); break;
        case WOp::AdjLeafUp:
        case WOp::AdjUpSchool:
        case WOp::AdjUpFused:
        case WOp::AdjDownSchool:
        case WOp::AdjDownFused:
        case WOp::AdjLeafDown:
            launch_worklist_adj(s.op, s.key, s.d_desc, s.d_tab, nctas, qn, q0, s.smem, f->stream);
            break;
        case WOp::AdjSpecReal:
        case WOp::AdjSpecUp:
        case WOp::AdjSpecDown: launch_worklist_vsp(s.op, s.d_desc, s.d_tab, nctas, qn, q0, s.smem, f->stream); break;
        default: launch_worklist_spec(s.op, s.d_desc, s.d_tab, nctas, qn, q0, s.smem, f->stream); break;
    }
    f->prof.end(f->stream);
    ++f->launches;
}

// the kernel sequence of one run (Q nodes in chunks of qc)
static void enqueue_run(Forest *f) {
    for (const WStep &s : f->pre) launch_step(f, s, 1, 0);
    for (int q0 = 0; q0 < f->Q; q0 += f->qc) {
        const int nq = std::min(f->qc, f->Q - q0);
        for (const WStep &s : f->steps) launch_step(f, s, nq, q0);
        if (f->vjp) {   // ordered sums over nodes: dL/dS shares and the roots' gbar
            launch_accum_strided((int)f->Ntot, nq, f->d_contrib, (size_t)f->Ntot, f->d_acc, q0 == 0, f->stream);
            launch_accum_strided((int)f->Rtot, nq, f->d_root, (size_t)f->Rtot, f->d_gradP, q0 == 0, f->stream);
            f->launches += 2;
            if (f->node_terms) {
                const size_t pq = (size_t)f->qc * f->Ntot, nodes = (size_t)f->tr.size() * f->Q;
                double *nA = f->d_part + 2 * pq;
                launch_node_reduce_members((int)f->tr.size(), f->d_mem, nq, (size_t)f->Ntot, f->d_part,
                                           f->d_part + pq, nA, nA + nodes, f->Q, q0, f->stream);
                ++f->launches;
            }
            continue;
        }
        launch_accumulate((int)f->Ntot, nq, f->d_contrib, f->d_acc, q0 == 0 ? 1 : 0, f->stream, &f->prof);
        ++f->launches;
    }
    launch_scatter((int)f->Ntot, f->d_acc, f->d_perm, nullptr, f->d_out, f->stream);
    ++f->launches;
}

// ------------------------------------------------------------ lifecycle
Forest *forest_create(int T, const int *n, const int *k, const double *S, std::string &err, bool vjp) {
    if (T < 1 || !n || !k || !S) { err = "invalid batch arguments"; return nullptr; }
    long tot = 0;
    std::vector<long> ioff(T + 1, 0), ipoff(T + 1, 0);
    for (int t = 0; t < T; ++t) {
        if (n[t] < 1 || k[t] < 1 || k[t] > n[t]) {
            err = "tournament " + std::to_string(t) + " needs 1 <= k <= n";
            return nullptr;
        }
        ioff[t + 1] = ioff[t] + n[t];
        ipoff[t + 1] = ipoff[t] + k[t];
        tot += n[t];
    }
    if (tot > (long)INT32_MAX / 2) { err = "batch too large (total players)"; return nullptr; }
    Forest *f = new Forest();
    f->vjp = vjp;
    f->T = T;
    f->ioff = ioff;
    f->ipoff = ipoff;
    f->n.assign(n, n + T);
    f->k.assign(k, k + T);
    // geometry of every tournament (sorts in parallel)
    std::vector<Plan *> all(T, nullptr);
    std::vector<std::string> errs(T);
    parallel_for(T, [&](int t) {
        Plan *p = new Plan();
        // adjoint forests: member trees under a single VJP plan's rules
        p->vjp = vjp;
        p->coeff_only = vjp && g_config.vjp_spectral_min_degree < 0;
        if (plan_geometry(p, n[t], S + ioff[t], k[t], errs[t]) != 0) {
            delete p;
            p = nullptr;
        } else if (vjp) {
            p->Lf = 0;   // every level's g is kept for the adjoint
        }
        all[t] = p;
    });
    for (int t = 0; t < T; ++t)
        if (!all[t]) {
            err = "tournament " + std::to_string(t) + ": " + errs[t];
            for (Plan *p : all) delete p;
            delete f;
            return nullptr;
        }
    for (int t = 0; t < T; ++t) {
        if (fits_worklist(all[t])) {
            f->tr.push_back(all[t]);
            f->tid.push_back(t);
        } else {
            delete all[t];
            f->fallback.push_back(t);
        }
    }
    for (int t : f->fallback) {   // own plans (own arenas and streams)
        if (vjp) {
            VjpPlan *v = vjp_plan_create(n[t], S + ioff[t], k[t], err);
            if (!v) {
                err = "tournament " + std::to_string(t) + ": " + err;
                forest_destroy(f);
                return nullptr;
            }
            f->fb_vjp.push_back(v);
            continue;
        }
        Plan *p = plan_create(n[t], S + ioff[t], k[t], nullptr, err);
        if (!p) {
            err = "tournament " + std::to_string(t) + ": " + err;
            forest_destroy(f);
            return nullptr;
        }
        f->fb_plans.push_back(p);
    }
    const int F = (int)f->tr.size();
    f->off.assign(F + 1, 0);
    f->poff.assign(F + 1, 0);
    for (int i = 0; i < F; ++i) {
        f->off[i + 1] = f->off[i] + f->tr[i]->n;
        f->poff[i + 1] = f->poff[i] + f->tr[i]->k;
    }
    f->Ntot = f->off[F];
    f->Ktot = f->poff[F];
    f->roff.assign(F + 1, 0);
    if (vjp)
        for (int i = 0; i < F; ++i) f->roff[i + 1] = f->roff[i] + ((f->tr[i]->k + 1) & ~1);
    f->Rtot = f->roff[F];
    f->compact = f->fallback.empty();

    cudaError_t e = cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { err = std::string("stream: ") + cudaGetErrorString(e); forest_destroy(f); return nullptr; }
    if (F == 0) return f;

    // node chunk from the memory budget
    size_t per_q = (size_t)2 * f->Ntot * 8 + 1024;
    for (Plan *p : f->tr)   // linear members keep checkpoints instead of a tree
        per_q += p->linear ? linear_ck_per_node(p->n, p->k) * sizeof(double) : p->tree_q_bytes;
    if (vjp) {   // adjoint buffers, the roots' gbar rows, node-term partials
        per_q += (size_t)f->Rtot * 8 + (size_t)2 * f->Ntot * 8;
        for (Plan *p : f->tr) per_q += vjp_level_layout(p, 1, nullptr, nullptr);
    }
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const size_t budget = g_config.max_device_bytes ? g_config.max_device_bytes
                                                    : std::min<size_t>((size_t)(free_b * 0.6), (size_t)64 << 30);
    int qc = (int)std::min<size_t>(256, std::max<size_t>(1, budget / std::max<size_t>(per_q, 1)));
    if (g_config.q_chunk > 0) qc = std::min(qc, g_config.q_chunk);
    f->qc = qc;

    // arena: shared arrays, then every tournament's tree buffers
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += align256(bytes); return o; };
    const size_t Nt = (size_t)f->Ntot;
    const size_t o_S = take(8 * Nt), o_perm = take(4 * Nt), o_pay = take(8 * (size_t)f->Ktot);
    const size_t o_acc = take(8 * Nt), o_out = take(8 * Nt);
    const size_t o_a = take(8 * Nt * qc), o_con = take(8 * Nt * qc);
    std::vector<size_t> o_tree(F), o_adj(F);
    for (int i = 0; i < F; ++i) {
        Plan *p = f->tr[i];
        o_tree[i] = p->linear ? take(sizeof(double) * (size_t)qc * linear_ck_per_node(p->n, p->k))
                              : take(plan_tree_layout(p, qc, nullptr));
    }
    size_t o_cot = 0, o_gp = 0, o_root = 0, o_mem = 0;
    if (vjp) {
        o_cot = take(8 * Nt);
        o_gp = take(8 * (size_t)f->Rtot);
        o_root = take(8 * (size_t)qc * f->Rtot);
        o_mem = take(sizeof(longlong2) * (size_t)F);
        for (int i = 0; i < F; ++i) o_adj[i] = take(vjp_level_layout(f->tr[i], qc, nullptr, nullptr));
    }
    e = dev_alloc((void **)&f->arena, off, f->stream, true);
    if (e != cudaSuccess) {
        err = "device allocation of " + std::to_string(off) + " bytes failed: " + cudaGetErrorString(e);
        forest_destroy(f);
        return nullptr;
    }
    f->arena_bytes = off;
    char *A = f->arena;
    f->d_S = (double *)(A + o_S);
    f->d_perm = (int *)(A + o_perm);
    f->d_payout = (double *)(A + o_pay);
    f->d_acc = (double *)(A + o_acc);
    f->d_out = (double *)(A + o_out);
    f->d_a = (double *)(A + o_a);
    f->d_contrib = (double *)(A + o_con);
    std::vector<double> hS(Nt);
    std::vector<int> hperm(Nt);
    int logNeed = 12;
    for (int i = 0; i < F; ++i) {
        Plan *p = f->tr[i];
        if (p->linear) p->d_ck = (double *)(A + o_tree[i]);
        else plan_tree_layout(p, qc, A + o_tree[i]);
        p->qc = qc;
        p->d_S = f->d_S + f->off[i];
        p->d_payout = f->d_payout + f->poff[i];
        for (int l = 1; l < p->L; ++l) {
            if (p->lv[l].fft) logNeed = std::max(logNeed, ilog2l(p->lv[l].fftn));
            if (p->lv[l].kind == 2) logNeed = std::max(logNeed, ilog2l(2 * p->lv[l].deg));
        }
    }
    parallel_for(F, [&](int i) {   // sorted stacks and the permutation, members side by side
        const Plan *p = f->tr[i];
        const long fo = f->off[i];
        for (int j = 0; j < p->n; ++j) {
            hS[fo + j] = p->S_sorted[j];
            hperm[fo + j] = (int)(fo + p->perm[j]);
        }
    });
    std::vector<longlong2> hmem;
    if (vjp) {
        f->d_cot = (double *)(A + o_cot);
        f->d_gradP = (double *)(A + o_gp);
        f->d_root = (double *)(A + o_root);
        f->d_mem = (longlong2 *)(A + o_mem);
        f->vb.assign(F, VjpBufs{});
        for (int i = 0; i < F; ++i) {
            Plan *p = f->tr[i];
            VjpBufs &b = f->vb[i];
            vjp_level_layout(p, qc, A + o_adj[i], &b);
            b.kst = (p->k + 1) & ~1;
            b.root = f->d_root + f->roff[i];   // rows of Rtot: every member's root gbar side by side
            b.root_q = (size_t)f->Rtot;
            b.cot = f->d_cot + f->off[i];
            b.a = f->d_a + f->off[i];
            b.aq = Nt;
            b.contrib = f->d_contrib + f->off[i];
            if (p->L == 1) {   // the single leaf block is the root: its gbar goes to the root rows
                b.gb[0] = b.root;
                b.gb_q[0] = b.root_q;
                b.gb_st[0] = b.kst;
            }
            hmem.push_back(make_longlong2(f->off[i], p->n));
        }
    }
    f->tw = twiddles(logNeed, f->stream, err, &f->logTW);
    if (!f->tw) { forest_destroy(f); return nullptr; }
    e = cudaMemcpyAsync(f->d_S, hS.data(), 8 * Nt, cudaMemcpyHostToDevice, f->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(f->d_perm, hperm.data(), 4 * Nt, cudaMemcpyHostToDevice, f->stream);
    if (e == cudaSuccess && vjp) {
        e = cudaMemcpyAsync(f->d_mem, hmem.data(), sizeof(longlong2) * F, cudaMemcpyHostToDevice, f->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(f->d_root, 0, 8 * (size_t)qc * f->Rtot, f->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(f->stream);
    if (e != cudaSuccess) { err = std::string("batch upload: ") + cudaGetErrorString(e); forest_destroy(f); return nullptr; }
    return f;
}

void forest_destroy(Forest *f) {
    if (!f) return;
    if (f->stream) cudaStreamSynchronize(f->stream);
    if (f->graph) cudaGraphExecDestroy(f->graph);
    if (f->d_desc) cudaFree(f->d_desc);
    if (f->d_node) cudaFree(f->d_node);
    if (f->d_part) cudaFree(f->d_part);
    if (f->arena) {
        cudaFreeAsync(f->arena, f->stream);
        cudaStreamSynchronize(f->stream);
    }
    if (f->ev0) cudaEventDestroy(f->ev0);
    if (f->ev1) cudaEventDestroy(f->ev1);
    for (cudaEvent_t ev : f->prof.pool) cudaEventDestroy(ev);
    if (f->stream) cudaStreamDestroy(f->stream);
    for (Plan *p : f->tr) delete p;   // geometry only: their buffers live in the forest arena
    for (Plan *p : f->fb_plans) plan_destroy(p);
    for (VjpPlan *v : f->fb_vjp) vjp_plan_destroy(v);
    delete f;
}

// nodes per tournament (its own Smax), node-major per tournament: [t][Q][3]
static int prepare_nodes(Forest *f, int Q, std::string &err) {
    const int F = (int)f->tr.size();
    std::vector<double> h((size_t)F * Q * 3);
    std::vector<int> hz((size_t)F * Q);
    parallel_for(F, [&](int i) {
        std::vector<double> logv, w;
        const Plan *p = f->tr[i];
        make_nodes(Q, p->Smax, logv, w);
        double *o = h.data() + (size_t)i * Q * 3;
        int *z = hz.data() + (size_t)i * Q;
        for (int q = 0; q < Q; ++q) {
            o[3 * q] = logv[q];
            o[3 * q + 1] = w[q];
            o[3 * q + 2] = std::exp(-logv[q]);
            z[q] = zero_prefix(p->S_sorted.data(), p->n, logv[q]);
        }
    });
    f->h_z = hz;
    if (f->d_node) cudaFree(f->d_node);
    f->d_node = nullptr;
    const size_t nb = sizeof(double) * h.size();
    cudaError_t e = dev_alloc((void **)&f->d_node, nb + sizeof(int) * hz.size(), f->stream, false);
    int *dz = e == cudaSuccess ? (int *)((char *)f->d_node + nb) : nullptr;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(f->d_node, h.data(), nb, cudaMemcpyHostToDevice, f->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dz, hz.data(), sizeof(int) * hz.size(), cudaMemcpyHostToDevice, f->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(f->stream);
    if (e != cudaSuccess) { err = std::string("node table: ") + cudaGetErrorString(e); return -1; }
    for (int i = 0; i < F; ++i) {
        f->tr[i]->d_node = f->d_node + (size_t)i * Q * 3;
        f->tr[i]->d_z = dz + (size_t)i * Q;
    }
    return 0;
}

// node tables, work lists and (adjoint forests with node terms) partials for
// Q nodes; the graph is recaptured when any of them changes
static int forest_prepare(Forest *f, int Q, bool node_terms, std::string &err) {
    if (Q == f->Q && node_terms == f->node_terms) return 0;
    if (f->graph) cudaGraphExecDestroy(f->graph);
    f->graph = nullptr;
    if (Q != f->Q) {
        f->Q = Q;
        if (prepare_nodes(f, Q, err) != 0) { f->Q = 0; return -1; }
    }
    f->node_terms = node_terms;
    if (f->vjp && node_terms) {
        const size_t need = 2 * (size_t)f->qc * f->Ntot + 2 * f->tr.size() * (size_t)Q;
        if (need > f->part_cap) {
            cudaStreamSynchronize(f->stream);
            if (f->d_part) cudaFree(f->d_part);
            f->d_part = nullptr;
            f->part_cap = 0;
            cudaError_t e = dev_alloc((void **)&f->d_part, sizeof(double) * need, f->stream, false);
            if (e != cudaSuccess) { err = std::string("node-term buffers: ") + cudaGetErrorString(e); f->Q = 0; return -1; }
            f->part_cap = need;
        }
    }
    build_steps(f);
    if (upload_steps(f, err) != 0) { f->Q = 0; return -1; }
    return 0;
}

// payouts in forest order
static int forest_upload_payout(Forest *f, const double *payout, std::string &err) {
    cudaError_t e;
    if (f->compact) {
        e = cudaMemcpyAsync(f->d_payout, payout, sizeof(double) * f->Ktot, cudaMemcpyHostToDevice, f->stream);
    } else {
        f->h_pay.resize(f->Ktot);
        for (size_t i = 0; i < f->tr.size(); ++i)
            memcpy(f->h_pay.data() + f->poff[i], payout + f->ipoff[f->tid[i]], sizeof(double) * f->tr[i]->k);
        e = cudaMemcpyAsync(f->d_payout, f->h_pay.data(), sizeof(double) * f->Ktot, cudaMemcpyHostToDevice,
                            f->stream);
    }
    if (e != cudaSuccess) { err = std::string("payout upload: ") + cudaGetErrorString(e); return -1; }
    return 0;
}

// the run's kernel sequence between two events: a graph replay, or direct
// launches when profiling
static int forest_launch(Forest *f, std::string &err) {
    cudaError_t e = cudaSuccess;
    if (!f->ev0) { cudaEventCreate(&f->ev0); cudaEventCreate(&f->ev1); }
    f->prof.used = 0;
    f->prof.recs.clear();
    const bool use_graph = f->graphs && !f->prof.on;
    if (use_graph && !f->graph) {   // capture the kernel sequence once per node count
        cudaGraph_t g = nullptr;
        f->launches = 0;
        e = cudaStreamBeginCapture(f->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            enqueue_run(f);
            e = cudaStreamEndCapture(f->stream, &g);
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&f->graph, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) { err = std::string("graph capture: ") + cudaGetErrorString(e); return -1; }
        f->graph_launches = f->launches;
    }
    cudaEventRecord(f->ev0, f->stream);
    if (use_graph) {
        e = cudaGraphLaunch(f->graph, f->stream);
        f->launches = f->graph_launches;
    } else {
        f->launches = 0;
        enqueue_run(f);
        e = cudaGetLastError();
    }
    cudaEventRecord(f->ev1, f->stream);
    if (e != cudaSuccess) { err = std::string("batch launch: ") + cudaGetErrorString(e); return -1; }
    return 0;
}

// device time of the run and, when profiling, the per-launch records
static void forest_collect(Forest *f) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, f->ev0, f->ev1);
    f->last_device_ms = ms;
    if (!f->prof.on) return;
    for (const ProfRec &r : f->prof.recs) {
        float ems = 0.f;
        cudaEventElapsedTime(&ems, r.a, r.b);
        Plan::KStat *ks = nullptr;
        for (auto &x : f->kstats)
            if (x.name == r.name) ks = &x;
        if (!ks) { f->kstats.push_back({r.name, 0.0, 0, 0.0}); ks = &f->kstats.back(); }
        ks->ms += ems;
        ks->launches += 1;
        ks->flops += r.flops;
    }
}

int forest_run(Forest *f, int Q, const double *payout, double *equity, IcmGpuRunStats *stats, std::string &err) {
    if (!f || Q < 1 || !payout || !equity) { err = "invalid arguments"; return -1; }
    if (f->vjp) { err = "this batch computes VJPs (use the VJP run)"; return -1; }
    const double t0 = now_ns();
    f->launches = 0;
    const int F = (int)f->tr.size();
    cudaError_t e = cudaSuccess;
    if (F > 0) {
        if (forest_prepare(f, Q, false, err) != 0) return -1;
        if (forest_upload_payout(f, payout, err) != 0) return -1;
        if (forest_launch(f, err) != 0) return -1;
        if (f->compact) {
            e = cudaMemcpyAsync(equity, f->d_out, sizeof(double) * f->Ntot, cudaMemcpyDeviceToHost, f->stream);
        } else {
            f->h_out.resize(f->Ntot);
            e = cudaMemcpyAsync(f->h_out.data(), f->d_out, sizeof(double) * f->Ntot, cudaMemcpyDeviceToHost,
                                f->stream);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(f->stream);
        if (e != cudaSuccess) { err = std::string("batch execution: ") + cudaGetErrorString(e); return -1; }
        if (!f->compact)
            for (int i = 0; i < F; ++i)
                memcpy(equity + f->ioff[f->tid[i]], f->h_out.data() + f->off[i], sizeof(double) * f->tr[i]->n);
        forest_collect(f);
    } else {
        f->last_device_ms = 0.0;
    }
    // tournaments beyond the one-CTA kernels: single plans
    for (size_t i = 0; i < f->fallback.size(); ++i) {
        const int t = f->fallback[i];
        Plan *p = f->fb_plans[i];
        if (plan_run(p, Q, payout + f->ipoff[t], equity + f->ioff[t], nullptr, err) != 0) return -1;
        f->launches += p->launches;
    }
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->total_ns = now_ns() - t0;
        stats->peak_vram_bytes = f->arena_bytes;
        stats->engine = 1;
    }
    return 0;
}

// Adjoint forest: per chunk of nodes the forward tree of every member (no
// divide), then the adjoint passes; dL/dS and the roots' gbar are summed over
// nodes in order, so each member's gradients equal its single-plan VJP's bit
// for bit.
int forest_vjp_run(Forest *f, int Q, const double *payout, const double *cot, int flags, double *grad_S,
                   double *grad_payout, IcmGpuRunStats *stats, std::string &err) {
    if (!f || Q < 1 || !payout || !cot || !grad_S || !grad_payout) { err = "invalid arguments"; return -1; }
    if (!f->vjp) { err = "this batch computes equities (use the batch run)"; return -1; }
    const double t0 = now_ns();
    const bool node_terms = (flags & 1) != 0;
    f->launches = 0;
    const int F = (int)f->tr.size();
    cudaError_t e = cudaSuccess;
    if (F > 0) {
        if (forest_prepare(f, Q, node_terms, err) != 0) return -1;
        if (forest_upload_payout(f, payout, err) != 0) return -1;
        // cotangents in each member's sorted order
        f->h_cot.resize(f->Ntot);
        for (int i = 0; i < F; ++i) {
            const Plan *p = f->tr[i];
            const double *c = cot + f->ioff[f->tid[i]];
            double *o = f->h_cot.data() + f->off[i];
            for (int j = 0; j < p->n; ++j) o[j] = c[p->perm[j]];
        }
        e = cudaMemcpyAsync(f->d_cot, f->h_cot.data(), sizeof(double) * f->Ntot, cudaMemcpyHostToDevice, f->stream);
        if (e != cudaSuccess) { err = std::string("cotangent upload: ") + cudaGetErrorString(e); return -1; }
        if (forest_launch(f, err) != 0) return -1;
        f->h_out.resize(f->Ntot);
        f->h_gp.resize(f->Rtot);
        double *gs = f->compact ? grad_S : f->h_out.data();
        e = cudaMemcpyAsync(gs, f->d_out, sizeof(double) * f->Ntot, cudaMemcpyDeviceToHost, f->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(f->h_gp.data(), f->d_gradP, sizeof(double) * f->Rtot, cudaMemcpyDeviceToHost,
                                f->stream);
        const size_t nodes = (size_t)F * Q;
        if (node_terms) {
            f->h_nodeA.resize(nodes);
            f->h_nodeB.resize(nodes);
            const double *nA = f->d_part + 2 * (size_t)f->qc * f->Ntot;
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(f->h_nodeA.data(), nA, sizeof(double) * nodes, cudaMemcpyDeviceToHost, f->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(f->h_nodeB.data(), nA + nodes, sizeof(double) * nodes, cudaMemcpyDeviceToHost,
                                    f->stream);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(f->stream);
        if (e != cudaSuccess) { err = std::string("batch execution: ") + cudaGetErrorString(e); return -1; }
        if (!f->compact)
            for (int i = 0; i < F; ++i)
                memcpy(grad_S + f->ioff[f->tid[i]], f->h_out.data() + f->off[i], sizeof(double) * f->tr[i]->n);
        for (int i = 0; i < F; ++i)
            memcpy(grad_payout + f->ipoff[f->tid[i]], f->h_gp.data() + f->roff[i], sizeof(double) * f->tr[i]->k);
        if (node_terms) {   // every node has a positive weight: all Q are active
            std::vector<int> qidx(Q);
            for (int q = 0; q < Q; ++q) qidx[q] = q;
            const std::vector<double> none;
            for (int i = 0; i < F; ++i) {
                const Plan *p = f->tr[i];
                const std::vector<double> A(f->h_nodeA.begin() + (size_t)i * Q, f->h_nodeA.begin() + (size_t)(i + 1) * Q);
                const std::vector<double> Bw(f->h_nodeB.begin() + (size_t)i * Q,
                                             f->h_nodeB.begin() + (size_t)(i + 1) * Q);
                grad_S[f->ioff[f->tid[i]] + p->perm[0]] += node_shift_term(Q, p->Smax, qidx, none, A, Bw);
            }
        }
        forest_collect(f);
    } else {
        f->last_device_ms = 0.0;
    }
    for (size_t i = 0; i < f->fallback.size(); ++i) {   // beyond the one-CTA kernels: single plans
        const int t = f->fallback[i];
        VjpPlan *v = f->fb_vjp[i];
        if (vjp_plan_run(v, Q, payout + f->ipoff[t], cot + f->ioff[t], grad_S + f->ioff[t],
                         grad_payout + f->ipoff[t], flags, nullptr, err) != 0)
            return -1;
        f->launches += v->p->launches;
    }
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->total_ns = now_ns() - t0;
        stats->peak_vram_bytes = f->arena_bytes;
        stats->engine = 1;
    }
    return 0;
}

}  // namespace icmg
