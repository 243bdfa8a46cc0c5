// host_mlp.cpp -- C ABI of the learned residual network (host buffers in and
// out), used to train it, to check its gradients and to run it standalone.
#include "gs_mlp.h"

#include <cstdio>
#include <memory>

using namespace gs;

struct gsgpu_mlp {
    MlpDevice dev;
    cudaStream_t stream = nullptr;
    DBuf feat, target, pred;
    ~gsgpu_mlp()
    {
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

int report(ErrorStatus st)
{
    if (st.return_code == GRAV_SUCCESS) return 0;
    const int rc = st.return_code;
    print_and_free_traceback(&st);
    return rc;
}

ErrorStatus stage(gsgpu_mlp *m, const float *h_feat, const float *h_target, int n)
{
    GS_TRY(m->feat.reserve((size_t)n * MLP_IN * sizeof(float)));
    GS_CUDA(cudaMemcpyAsync(m->feat.p, h_feat, (size_t)n * MLP_IN * sizeof(float),
                            cudaMemcpyHostToDevice, m->stream));
    if (h_target) {
        GS_TRY(m->target.reserve((size_t)n * MLP_OUT * sizeof(float)));
        GS_CUDA(cudaMemcpyAsync(m->target.p, h_target, (size_t)n * MLP_OUT * sizeof(float),
                                cudaMemcpyHostToDevice, m->stream));
    }
    return ok();
}

}  // namespace

extern "C" {

int gsgpu_mlp_num_params(void) { return MLP_NPARAM; }

int gsgpu_mlp_create(gsgpu_mlp **out, unsigned long long seed)
{
    if (!out) return GRAV_POINTER_ERROR;
    const DeviceInfo *d = nullptr;
    int rc = report(device_info(&d));
    if (rc) return rc;
    std::unique_ptr<gsgpu_mlp> m(new gsgpu_mlp());
    if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess)
        return GRAV_FAILURE;
    rc = report(m->dev.setup(seed, m->stream));
    if (rc) return rc;
    *out = m.release();
    return 0;
}

void gsgpu_mlp_destroy(gsgpu_mlp *m) { delete m; }

int gsgpu_mlp_get_params(gsgpu_mlp *m, float *h)
{
    if (!m || !h) return GRAV_POINTER_ERROR;
    if (cudaMemcpyAsync(h, m->dev.params.p, MLP_NPARAM * sizeof(float), cudaMemcpyDeviceToHost,
                        m->stream) != cudaSuccess ||
        cudaStreamSynchronize(m->stream) != cudaSuccess)
        return GRAV_FAILURE;
    return 0;
}

int gsgpu_mlp_set_params(gsgpu_mlp *m, const float *h)
{
    if (!m || !h) return GRAV_POINTER_ERROR;
    if (cudaMemcpyAsync(m->dev.params.p, h, MLP_NPARAM * sizeof(float), cudaMemcpyHostToDevice,
                        m->stream) != cudaSuccess ||
        cudaStreamSynchronize(m->stream) != cudaSuccess)
        return GRAV_FAILURE;
    return 0;
}

int gsgpu_mlp_forward(gsgpu_mlp *m, const float *h_feat, int n, float *h_pred)
{
    if (!m || !h_feat || !h_pred) return GRAV_POINTER_ERROR;
    if (n <= 0) return GRAV_VALUE_ERROR;
    int rc = report(stage(m, h_feat, nullptr, n));
    if (!rc) rc = report(m->pred.reserve((size_t)n * MLP_OUT * sizeof(float)));
    if (!rc) rc = report(m->dev.forward(m->feat.as<float>(), n, m->pred.as<float>(), m->stream));
    if (rc) return rc;
    if (cudaMemcpyAsync(h_pred, m->pred.p, (size_t)n * MLP_OUT * sizeof(float),
                        cudaMemcpyDeviceToHost, m->stream) != cudaSuccess)
        return GRAV_FAILURE;
    return report(m->dev.check(m->stream));
}

int gsgpu_mlp_gradients(gsgpu_mlp *m, const float *h_feat, const float *h_target, int n,
                        float *h_grad, double *loss_sum)
{
    if (!m || !h_feat || !h_target || !h_grad) return GRAV_POINTER_ERROR;
    if (n <= 0) return GRAV_VALUE_ERROR;
    int rc = report(stage(m, h_feat, h_target, n));
    if (!rc) rc = report(m->dev.gradients(m->feat.as<float>(), m->target.as<float>(), n, m->stream));
    if (rc) return rc;
    if (cudaMemcpyAsync(h_grad, m->dev.grads.p, MLP_NPARAM * sizeof(float), cudaMemcpyDeviceToHost,
                        m->stream) != cudaSuccess ||
        cudaMemsetAsync(m->dev.grads.p, 0, MLP_NPARAM * sizeof(float), m->stream) != cudaSuccess)
        return GRAV_FAILURE;
    double l = 0.0;
    rc = report(m->dev.read_loss(m->stream, &l));
    if (loss_sum) *loss_sum = l;
    if (!rc) rc = report(m->dev.check(m->stream));
    return rc;
}

int gsgpu_mlp_train_step(gsgpu_mlp *m, const float *h_feat, const float *h_target, int n, float lr,
                         double *loss_sum)
{
    if (!m || !h_feat || !h_target) return GRAV_POINTER_ERROR;
    if (n <= 0) return GRAV_VALUE_ERROR;
    int rc = report(stage(m, h_feat, h_target, n));
    if (!rc)
        rc = report(m->dev.train_step(m->feat.as<float>(), m->target.as<float>(), n, lr, m->stream));
    if (rc) return rc;
    double l = 0.0;
    rc = report(m->dev.read_loss(m->stream, &l));
    if (loss_sum) *loss_sum = l;
    if (!rc) rc = report(m->dev.check(m->stream));
    return rc;
}

}  // extern "C"
