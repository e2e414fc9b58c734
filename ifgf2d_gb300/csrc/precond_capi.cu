// precond_capi.cu -- the learned right preconditioner behind the C ABI: the network object,
// training steps on the GPU, gradients for the tests, and its application to residuals.
//
// The reference has no preconditioner (opGMRES runs unpreconditioned, ForwardMap.tpp:673-690);
// this net and the flexible GMRES that uses it (ifgf2d_solve_fgmres) are additions.
#include "context.hpp"
#include "precond_net.cuh"

#include <cmath>
#include <random>
#include <vector>

using namespace ifgf;

struct ifgf2d_net {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    long long off_w[kNetLayers] = {0}, off_b[kNetLayers] = {0}, nparam = 0;
    DBuf<float> p, g, m, v, zero_bias;
    DBuf<__nv_bfloat16> Wt[kNetLayers], Wb[kNetLayers];
    int step = 0;
    // 1: the output is the correction weighted by the operator's flat symbol magnitude |sigma|
    // (trained on Op(|sigma|) e targets); the preconditioner applies Op(1/|sigma|) to it
    int weighted = 0;
    // batch workspace for `rows_cap` padded rows, `pts_cap` points, `seg_cap` samples
    long long rows_cap = 0, pts_cap = 0;
    int seg_cap = 0;
    DBuf<__nv_bfloat16> X[kNetLayers], Y[kNetLayers], gbf;
    DBuf<float> O, T, gO, G, dpre, dX, part, sigma;
    DBuf<double> loss;
    DBuf<int> kerr;                 // set by a convolution whose bounded tensor-core wait ran out
    DBuf<double2> r, e, z;
    DBuf<double4> geom;
    DBuf<double> kseg;
    DBuf<int> seg_start, seg_len, seg_pt, pt_row, pt_seg;
    // the batch currently laid out in the index arrays
    int nseg = 0;
    long long rows = 0, npts = 0;
    std::vector<int> cur_len;
};

#define NK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            net->err = std::string(#call) + ": " + cudaGetErrorString(e_);                \
            return IFGF2D_ERR_CUDA;                                                       \
        }                                                                                 \
    } while (0)

namespace {

long long layer_w(int l) { return (long long)net_cout(l) * kNetTaps * net_cin(l); }

int net_pack(ifgf2d_net* net, cudaStream_t s) {
    for (int l = 0; l < kNetLayers; ++l)
        launch_net_pack(net->p.p + net->off_w[l], net_cin(l), net_cout(l), net->Wt[l].p, net->Wb[l].p, s);
    NK(cudaGetLastError());
    return IFGF2D_OK;
}

// lay out a batch: sample s occupies rows [start - 3, start + len + 3)
int net_layout(ifgf2d_net* net, int nseg, const int* len) {
    long long npts = 0, rows = 0;
    for (int s = 0; s < nseg; ++s) {
        if (len[s] < 2 * kHalo) { net->err = "each sample needs at least 6 points"; return IFGF2D_ERR_ARG; }
        npts += len[s]; rows += len[s] + 2 * kHalo;
    }
    const bool same = nseg == net->nseg && std::equal(len, len + nseg, net->cur_len.begin(), net->cur_len.end());
    if (same) return IFGF2D_OK;
    if (rows > net->rows_cap) {
        for (int l = 0; l < kNetLayers; ++l) {
            NK(net->X[l].alloc((size_t)rows * (l == 0 ? kNetInPad : kNetHidden)));
            NK(net->Y[l].alloc((size_t)rows * kNetHidden));
        }
        NK(net->gbf.alloc((size_t)rows * kNetHidden));
        NK(net->O.alloc((size_t)rows * kNetOutPad)); NK(net->gO.alloc((size_t)rows * kNetOutPad));
        NK(net->T.alloc((size_t)rows * 2));
        NK(net->G.alloc((size_t)rows * kNetHidden)); NK(net->dpre.alloc((size_t)rows * kNetHidden));
        NK(net->dX.alloc((size_t)rows * kNetHidden));
        NK(net->part.alloc((size_t)conv_wgrad_chunks((int)rows) * (kNetHidden * kNetTaps * kNetHidden + kNetHidden)));
        net->rows_cap = rows;
    }
    if (npts > net->pts_cap) {
        NK(net->r.alloc(npts)); NK(net->e.alloc(npts)); NK(net->z.alloc(npts)); NK(net->geom.alloc(npts));
        NK(net->pt_row.alloc(npts)); NK(net->pt_seg.alloc(npts));
        net->pts_cap = npts;
    }
    if (nseg > net->seg_cap) {
        NK(net->seg_start.alloc(nseg)); NK(net->seg_len.alloc(nseg)); NK(net->seg_pt.alloc(nseg));
        NK(net->sigma.alloc(3 * (size_t)nseg)); NK(net->kseg.alloc(nseg));
        net->seg_cap = nseg;
    }
    std::vector<int> st(nseg), pt(nseg), prow(npts), pseg(npts);
    long long rr = 0, pp = 0;
    for (int s = 0; s < nseg; ++s) {
        st[s] = (int)(rr + kHalo); pt[s] = (int)pp;
        for (int i = 0; i < len[s]; ++i) { prow[pp + i] = st[s] + i; pseg[pp + i] = s; }
        rr += len[s] + 2 * kHalo; pp += len[s];
    }
    cudaStream_t s = net->stream;
    NK(cudaMemcpyAsync(net->seg_start.p, st.data(), sizeof(int) * nseg, cudaMemcpyHostToDevice, s));
    NK(cudaMemcpyAsync(net->seg_len.p, len, sizeof(int) * nseg, cudaMemcpyHostToDevice, s));
    NK(cudaMemcpyAsync(net->seg_pt.p, pt.data(), sizeof(int) * nseg, cudaMemcpyHostToDevice, s));
    NK(cudaMemcpyAsync(net->pt_row.p, prow.data(), sizeof(int) * npts, cudaMemcpyHostToDevice, s));
    NK(cudaMemcpyAsync(net->pt_seg.p, pseg.data(), sizeof(int) * npts, cudaMemcpyHostToDevice, s));
    NK(cudaStreamSynchronize(s));
    net->nseg = nseg; net->rows = rows; net->npts = npts;
    net->cur_len.assign(len, len + nseg);
    return IFGF2D_OK;
}

// forward pass from the residuals in net->r (features, six layers, output O);
// keep_relu: store each hidden layer's ReLU output in Y for the backward pass
void net_forward(ifgf2d_net* net, const double2* r, const double4* geom, bool keep_relu, cudaStream_t s) {
    const long long R = net->rows;
    launch_seg_rms(r, net->seg_pt.p, net->seg_len.p, net->nseg, net->sigma.p, s);
    cudaMemsetAsync(net->X[0].p, 0, sizeof(__nv_bfloat16) * R * kNetInPad, s);
    launch_features(r, geom, net->kseg.p, net->sigma.p, net->pt_row.p, net->pt_seg.p, (int)net->npts, net->X[0].p, s);
    launch_halo(net->X[0].p, kNetInPad, net->seg_start.p, net->seg_len.p, net->nseg, s);
    const float* p = net->p.p;
    launch_conv_fwd(net->X[0].p, (int)R, kNetInPad, net->Wt[0].p, p + net->off_b[0], kNetHidden, true, false, net->X[1].p,
                    nullptr, net->kerr.p, s);
    launch_halo(net->X[1].p, kNetHidden, net->seg_start.p, net->seg_len.p, net->nseg, s);
    for (int l = 1; l < kNetLayers - 1; ++l) {
        if (keep_relu) {
            launch_conv_fwd(net->X[l].p, (int)R, kNetHidden, net->Wt[l].p, p + net->off_b[l], kNetHidden, true, false, net->Y[l].p,
                            nullptr, net->kerr.p, s);
            launch_add_bf(net->Y[l].p, net->X[l].p, R * kNetHidden, net->X[l + 1].p, s);
        } else {
            launch_conv_fwd(net->X[l].p, (int)R, kNetHidden, net->Wt[l].p, p + net->off_b[l], kNetHidden, true, true,
                            net->X[l + 1].p, nullptr, net->kerr.p, s);
        }
        launch_halo(net->X[l + 1].p, kNetHidden, net->seg_start.p, net->seg_len.p, net->nseg, s);
    }
    const int L = kNetLayers - 1;
    launch_conv_fwd(net->X[L].p, (int)R, kNetHidden, net->Wt[L].p, p + net->off_b[L], kNetOutPad, false, false, nullptr, net->O.p, net->kerr.p,
                    s);
}

// loss against the targets of net->e and the full backward pass into net->g
void net_backward(ifgf2d_net* net, cudaStream_t s) {
    const long long R = net->rows;
    const int np = (int)net->npts;
    cudaMemsetAsync(net->gO.p, 0, sizeof(float) * R * kNetOutPad, s);
    cudaMemsetAsync(net->loss.p, 0, sizeof(double), s);
    launch_targets(net->r.p, net->e.p, net->sigma.p, net->pt_row.p, net->pt_seg.p, np, net->T.p, s);
    launch_mse(net->O.p, net->T.p, net->pt_row.p, np, net->gO.p, net->loss.p, s);
    float* g = net->g.p;
    const int L = kNetLayers - 1;
    launch_conv_wgrad(net->X[L].p, net->gO.p, nullptr, (int)R, kNetHidden, kNetOutPad, net->part.p, g + net->off_w[L],
                      g + net->off_b[L], s);
    launch_f2bf(net->gO.p, R * kNetOutPad, net->gbf.p, s);
    launch_conv_fwd(net->gbf.p, (int)R, kNetOutPad, net->Wb[L].p, net->zero_bias.p, kNetHidden, false, false, nullptr, net->G.p, net->kerr.p, s);
    launch_halo_fold(net->G.p, kNetHidden, net->seg_start.p, net->seg_len.p, net->nseg, s);
    for (int l = L - 1; l >= 1; --l) {
        // X[l+1] = relu(conv_l(X[l])) + X[l]: G holds dL/dX[l+1]
        launch_relu_grad(net->G.p, net->Y[l].p, R * kNetHidden, net->dpre.p, net->gbf.p, s);
        launch_conv_wgrad(net->X[l].p, net->dpre.p, nullptr, (int)R, kNetHidden, kNetHidden, net->part.p, g + net->off_w[l],
                          g + net->off_b[l], s);
        launch_conv_fwd(net->gbf.p, (int)R, kNetHidden, net->Wb[l].p, net->zero_bias.p, kNetHidden, false, false, nullptr,
                        net->dX.p, net->kerr.p, s);
        launch_halo_fold(net->dX.p, kNetHidden, net->seg_start.p, net->seg_len.p, net->nseg, s);
        launch_axpy_f(net->dX.p, R * kNetHidden, net->G.p, s);
    }
    launch_relu_grad(net->G.p, net->X[1].p, R * kNetHidden, net->dpre.p, net->gbf.p, s);
    launch_conv_wgrad(net->X[0].p, net->dpre.p, nullptr, (int)R, kNetInPad, kNetHidden, net->part.p, g + net->off_w[0],
                      g + net->off_b[0], s);
}

int net_stage(ifgf2d_net* net, int nseg, const int* len, const double* r, const double* e, const double* geom, const double* k) {
    if (!net || nseg <= 0 || !len || !r || !geom || !k) return IFGF2D_ERR_ARG;
    int rc = net_layout(net, nseg, len);
    if (rc != IFGF2D_OK) return rc;
    cudaStream_t s = net->stream;
    NK(cudaMemcpyAsync(net->r.p, r, sizeof(double2) * net->npts, cudaMemcpyHostToDevice, s));
    if (e) NK(cudaMemcpyAsync(net->e.p, e, sizeof(double2) * net->npts, cudaMemcpyHostToDevice, s));
    NK(cudaMemcpyAsync(net->geom.p, geom, sizeof(double4) * net->npts, cudaMemcpyHostToDevice, s));
    NK(cudaMemcpyAsync(net->kseg.p, k, sizeof(double) * nseg, cudaMemcpyHostToDevice, s));
    return IFGF2D_OK;
}

// after a synchronisation: did a convolution give up waiting for its tensor-core MMAs?
int net_check_kerr(ifgf2d_net* net) {
    int v = 0;
    NK(cudaMemcpy(&v, net->kerr.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (!v) return IFGF2D_OK;
    NK(cudaMemset(net->kerr.p, 0, sizeof(int)));
    net->err = "network convolution: a tensor-core completion wait ran out";
    return IFGF2D_ERR_CUDA;
}

}  // namespace

int ifgf::net_prepare_single(ifgf2d_net* net, long long N, const double* geom_host, double k, std::string& err) {
    AllocStream guard(nullptr);   // the network's buffers belong to its own stream: plain allocations
    if (!net || N <= 0 || N > (1LL << 30)) { err = "learned preconditioner: bad network or size"; return IFGF2D_ERR_ARG; }
    const int len = (int)N;
    int rc = net_layout(net, 1, &len);
    if (rc != IFGF2D_OK) { err = net->err; return rc; }
    if (cudaMemcpy(net->geom.p, geom_host, sizeof(double4) * N, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(net->kseg.p, &k, sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
        err = "learned preconditioner: upload failed";
        return IFGF2D_ERR_CUDA;
    }
    return IFGF2D_OK;
}
int ifgf::net_kernel_error(ifgf2d_net* net) { return net_check_kerr(net); }
bool ifgf::net_weighted(const ifgf2d_net* net) { return net && net->weighted; }
void ifgf::net_precondition_launch(ifgf2d_net* net, const double2* r, double2* z, cudaStream_t s) {
    net_forward(net, r, net->geom.p, false, s);
    launch_combine(r, net->O.p, net->sigma.p, net->pt_row.p, net->pt_seg.p, (int)net->npts, z, s);
}

// ------------------------------------------------------------------ C ABI
extern "C" long long ifgf2d_net_num_params(void) {
    long long n = 0;
    for (int l = 0; l < kNetLayers; ++l) n += layer_w(l) + net_cout(l);
    return n;
}

extern "C" int ifgf2d_net_create(unsigned long long seed, ifgf2d_net** out) {
    if (!out) return IFGF2D_ERR_ARG;
    *out = nullptr;
    ifgf2d_net* net = new ifgf2d_net;
    auto bad = [&](cudaError_t e) { if (e != cudaSuccess) { delete net; return true; } return false; };
    if (bad(cudaGetDevice(&net->device)) || bad(cudaStreamCreateWithFlags(&net->stream, cudaStreamNonBlocking)) ||
        bad(conv_init_attributes()))
        return IFGF2D_ERR_CUDA;
    long long off = 0;
    for (int l = 0; l < kNetLayers; ++l) { net->off_w[l] = off; off += layer_w(l); net->off_b[l] = off; off += net_cout(l); }
    net->nparam = off;
    // He initialisation over the real fan-in; padded channels zero; the output layer zero, so
    // the untrained preconditioner is the identity
    std::vector<float> h((size_t)off, 0.f);
    std::mt19937_64 rng(seed);
    for (int l = 0; l < kNetLayers - 1; ++l) {
        const int cin = net_cin(l), cout = net_cout(l), cin_real = l == 0 ? kNetFeatures : kNetHidden;
        const double sd = std::sqrt(2.0 / (kNetTaps * cin_real)) * (l == 0 ? 1.0 : 0.5);
        std::normal_distribution<double> nd(0.0, sd);
        for (int co = 0; co < cout; ++co)
            for (int tap = 0; tap < kNetTaps; ++tap)
                for (int ci = 0; ci < cin_real; ++ci) h[net->off_w[l] + ((long long)co * kNetTaps + tap) * cin + ci] = (float)nd(rng);
    }
    if (bad(net->p.upload(h)) || bad(net->g.alloc(off)) || bad(net->m.alloc(off)) || bad(net->v.alloc(off)) ||
        bad(net->zero_bias.alloc(kNetHidden)) || bad(net->loss.alloc(1)) || bad(net->kerr.alloc(1)))
        return IFGF2D_ERR_CUDA;
    cudaMemsetAsync(net->kerr.p, 0, sizeof(int), net->stream);
    cudaMemsetAsync(net->m.p, 0, sizeof(float) * off, net->stream);
    cudaMemsetAsync(net->v.p, 0, sizeof(float) * off, net->stream);
    cudaMemsetAsync(net->zero_bias.p, 0, sizeof(float) * kNetHidden, net->stream);
    for (int l = 0; l < kNetLayers; ++l) {
        if (bad(net->Wt[l].alloc(layer_w(l))) || bad(net->Wb[l].alloc(layer_w(l)))) return IFGF2D_ERR_CUDA;
    }
    if (net_pack(net, net->stream) != IFGF2D_OK || bad(cudaStreamSynchronize(net->stream))) { delete net; return IFGF2D_ERR_CUDA; }
    *out = net;
    return IFGF2D_OK;
}

extern "C" int ifgf2d_net_destroy(ifgf2d_net* net) {
    if (!net) return IFGF2D_ERR_ARG;
    if (net->stream) { cudaStreamSynchronize(net->stream); cudaStreamDestroy(net->stream); }
    delete net;
    return IFGF2D_OK;
}

extern "C" const char* ifgf2d_net_last_error(const ifgf2d_net* net) { return net ? net->err.c_str() : "null network"; }

extern "C" int ifgf2d_net_set_output_weighting(ifgf2d_net* net, int weighted) {
    if (!net || (weighted != 0 && weighted != 1)) return IFGF2D_ERR_ARG;
    net->weighted = weighted;
    return IFGF2D_OK;
}
extern "C" int ifgf2d_net_output_weighting(const ifgf2d_net* net) { return net ? net->weighted : -1; }

extern "C" int ifgf2d_net_get_params(ifgf2d_net* net, float* out) {
    if (!net || !out) return IFGF2D_ERR_ARG;
    NK(cudaStreamSynchronize(net->stream));
    NK(cudaMemcpy(out, net->p.p, sizeof(float) * net->nparam, cudaMemcpyDeviceToHost));
    return IFGF2D_OK;
}

extern "C" int ifgf2d_net_set_params(ifgf2d_net* net, const float* in) {
    if (!net || !in) return IFGF2D_ERR_ARG;
    NK(cudaStreamSynchronize(net->stream));
    NK(cudaMemcpy(net->p.p, in, sizeof(float) * net->nparam, cudaMemcpyHostToDevice));
    cudaMemsetAsync(net->m.p, 0, sizeof(float) * net->nparam, net->stream);
    cudaMemsetAsync(net->v.p, 0, sizeof(float) * net->nparam, net->stream);
    net->step = 0;
    int rc = net_pack(net, net->stream);
    if (rc != IFGF2D_OK) return rc;
    NK(cudaStreamSynchronize(net->stream));
    return IFGF2D_OK;
}

extern "C" int ifgf2d_net_gradient(ifgf2d_net* net, int nseg, const int* len, const double* r, const double* e, const double* geom,
                                   const double* k, double* loss, float* grad) {
    if (!e || !loss) return IFGF2D_ERR_ARG;
    int rc = net_stage(net, nseg, len, r, e, geom, k);
    if (rc != IFGF2D_OK) return rc;
    cudaStream_t s = net->stream;
    net_forward(net, net->r.p, net->geom.p, true, s);
    net_backward(net, s);
    NK(cudaGetLastError());
    NK(cudaMemcpyAsync(loss, net->loss.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    if (grad) NK(cudaMemcpyAsync(grad, net->g.p, sizeof(float) * net->nparam, cudaMemcpyDeviceToHost, s));
    NK(cudaStreamSynchronize(s));
    return net_check_kerr(net);
}

extern "C" int ifgf2d_net_train_step(ifgf2d_net* net, int nseg, const int* len, const double* r, const double* e, const double* geom,
                                     const double* k, float lr, float weight_decay, double* loss) {
    if (!e) return IFGF2D_ERR_ARG;
    int rc = net_stage(net, nseg, len, r, e, geom, k);
    if (rc != IFGF2D_OK) return rc;
    cudaStream_t s = net->stream;
    net_forward(net, net->r.p, net->geom.p, true, s);
    net_backward(net, s);
    launch_adamw(net->p.p, net->g.p, net->m.p, net->v.p, net->nparam, lr, 0.9f, 0.999f, 1e-8f, weight_decay, ++net->step, s);
    if ((rc = net_pack(net, s))) return rc;
    NK(cudaGetLastError());
    if (loss) NK(cudaMemcpyAsync(loss, net->loss.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    NK(cudaStreamSynchronize(s));
    return net_check_kerr(net);
}

extern "C" int ifgf2d_net_apply(ifgf2d_net* net, int nseg, const int* len, const double* r, const double* geom, const double* k,
                                double* z, float* out2) {
    if (!z && !out2) return IFGF2D_ERR_ARG;
    int rc = net_stage(net, nseg, len, r, nullptr, geom, k);
    if (rc != IFGF2D_OK) return rc;
    cudaStream_t s = net->stream;
    net_forward(net, net->r.p, net->geom.p, false, s);
    if (z) {
        launch_combine(net->r.p, net->O.p, net->sigma.p, net->pt_row.p, net->pt_seg.p, (int)net->npts, net->z.p, s);
        NK(cudaMemcpyAsync(z, net->z.p, sizeof(double2) * net->npts, cudaMemcpyDeviceToHost, s));
    }
    NK(cudaGetLastError());
    if (out2) {   // the raw two output channels per point, for the tests
        std::vector<float> O((size_t)net->rows * kNetOutPad);
        NK(cudaMemcpyAsync(O.data(), net->O.p, sizeof(float) * O.size(), cudaMemcpyDeviceToHost, s));
        NK(cudaStreamSynchronize(s));
        long long p = 0, row = 0;
        for (int sg = 0; sg < nseg; ++sg) {
            row += kHalo;
            for (int i = 0; i < len[sg]; ++i, ++p, ++row) { out2[2 * p] = O[row * kNetOutPad]; out2[2 * p + 1] = O[row * kNetOutPad + 1]; }
            row += kHalo;
        }
    }
    NK(cudaStreamSynchronize(s));
    return net_check_kerr(net);
}

// per point of the context, patch order: curvature, unit tangent (x, y), quadrature weight
extern "C" int ifgf2d_get_geometry_features(const ifgf2d_ctx* ctx, double* geom) {
    if (!ctx || !geom) return IFGF2D_ERR_ARG;
    const Discretisation& D = ctx->D;
    for (long long i = 0; i < D.N; ++i) {
        geom[4 * i] = D.kappa[i];
        geom[4 * i + 1] = -D.ny[i];   // tangent = (x', y') / |x'| with the normal (y', -x') / |x'|
        geom[4 * i + 2] = D.nx[i];
        geom[4 * i + 3] = D.wq[i];
    }
    return IFGF2D_OK;
}
