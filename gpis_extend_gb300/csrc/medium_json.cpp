// medium_json.cpp -- gpis_medium_desc_from_json: the "sparse_conv_noise" medium
// keys of a Tungsten scene (SparseConvolutionNoiseMedium::fromJson,
// SparseConvolutionNoiseMedium.cpp:102-118; GaussianProcessMedium::fromJson,
// GaussianProcessMedium.cpp:98-127; GaussianProcess::fromJson,
// GaussianProcess.cpp:173-184; SquaredExponentialCovariance::fromJson,
// GPFunctions.cpp:657-685; the mean factory, GaussianProcessFactory.cpp:14-22).
//
// Accepted "gaussian_process" shapes: {"type":"standard","mean":{...},
// "covariance":{...}} with means "spherical", "homogeneous", "linear" and
// "torus" (a torus about the y axis), and {"type":"csg","left":{torus GP},
// "right":{linear GP with direction (0,1,0)}} for the torus-union-plane field.
// Covariances: "squared_exponential" and "proc_nonstationary" wrapping one.
#include <cmath>
#include <string>

#include "../../include/gpis.h"
#include "json_lite.hpp"

namespace {

using gpis::json::Value;

struct Err {
    int code;
    std::string msg;
};

[[noreturn]] void bad(int code, const std::string &m) { throw Err{code, m}; }

double num(const Value &v, const char *key)
{
    if (v.kind == Value::Number) return v.num;
    if (v.kind == Value::Bool) return v.b ? 1.0 : 0.0;
    bad(GPIS_EINVAL, std::string("field '") + key + "' must be a number");
}

template <class T>
void field(const Value &o, const char *key, T &out)
{
    if (const Value *v = o.get(key)) out = (T)num(*v, key);
}

void vec3(const Value &o, const char *key, float *out)
{
    const Value *v = o.get(key);
    if (!v) return;
    if (v->kind == Value::Number) {
        out[0] = out[1] = out[2] = (float)v->num;
        return;
    }
    if (v->kind != Value::Array || v->arr.size() != 3) bad(GPIS_EINVAL, std::string("'") + key + "' must be a 3-vector");
    for (int i = 0; i < 3; ++i) out[i] = (float)num(v->arr[(size_t)i], key);
}

std::string str(const Value &o, const char *key, const std::string &dflt)
{
    const Value *v = o.get(key);
    if (!v) return dflt;
    if (v->kind != Value::String) bad(GPIS_EINVAL, std::string("'") + key + "' must be a string");
    return v->str;
}

uint32_t context_of(const std::string &s)
{
    if (s == "global") return GPIS_CTX_GLOBAL;
    if (s == "renewal+") return GPIS_CTX_RENEWAL_PLUS;
    if (s == "renewal") return GPIS_CTX_RENEWAL;
    if (s == "none") return GPIS_CTX_NONE;
    bad(GPIS_EINVAL, "Invalid correlation context: '" + s + "'");
}

uint32_t scheme_of(const std::string &s)
{
    if (s == "uni" || s == "UNI") return GPIS_SCHEME_UNI;
    if (s == "nee" || s == "NEE") return GPIS_SCHEME_NEE;
    if (s == "mis" || s == "MIS") return GPIS_SCHEME_MIS;
    bad(GPIS_EINVAL, "Invalid sparse conv sampling scheme: '" + s + "'");
}

void covariance(const Value &c, gpis_medium_desc *d)
{
    const std::string type = str(c, "type", "squared_exponential");
    if (type == "proc_nonstationary") {
        const Value *inner = c.get("cov");
        if (!inner) bad(GPIS_EINVAL, "proc_nonstationary needs 'cov'");
        covariance(*inner, d);
        if (const Value *mr = c.get("multiResolutionGrid")) d->multires = num(*mr, "multiResolutionGrid") != 0.0;
        if (const Value *ls = c.get("ls")) {
            // procedural vector a + b*sin(fx*x)*cos(fz*z) with its supremum
            d->ls_kind = GPIS_LS_SINCOS;
            float p[4] = {1.0f, 0.0f, 0.0f, 0.0f};
            field(*ls, "a", p[0]);
            field(*ls, "b", p[1]);
            field(*ls, "fx", p[2]);
            field(*ls, "fz", p[3]);
            for (int i = 0; i < 4; ++i) d->ls_params[i] = p[i];
            d->ls_max = std::fabs(p[0]) + std::fabs(p[1]);
            field(*ls, "max", d->ls_max);
        }
        return;
    }
    if (type != "squared_exponential") bad(GPIS_ENOTSUP, "covariance '" + type + "' is not supported");
    field(c, "sigma", d->sigma);
    field(c, "lengthScale", d->length_scale);
    vec3(c, "aniso", d->aniso);
    field(c, "localScale", d->kernel_scale);
    if (const Value *u = c.get("useAnisoMtx"))
        if (num(*u, "useAnisoMtx") != 0.0) bad(GPIS_ENOTSUP, "matrix anisotropy is not supported");
}

void mean(const Value &m, gpis_medium_desc *d)
{
    const std::string type = str(m, "type", "spherical");
    if (type == "spherical") {
        d->mean_kind = GPIS_MEAN_SPHERE;
        float c[3] = {0, 0, 0}, r = 1.0f;
        vec3(m, "center", c);
        field(m, "radius", r);
        d->mean_params[0] = c[0]; d->mean_params[1] = c[1]; d->mean_params[2] = c[2]; d->mean_params[3] = r;
    } else if (type == "homogeneous") {
        d->mean_kind = GPIS_MEAN_HOMOGENEOUS;
        float off = 0.0f;
        field(m, "offset", off);
        d->mean_params[0] = off;
    } else if (type == "linear") {
        // mean = dot(p - ref, normalize(dir)) * scale (LinearMean, GPFunctions.hpp:1008-1045)
        float ref[3] = {0, 0, 0}, dir[3] = {1, 0, 0}, scale = 1.0f;
        vec3(m, "reference_point", ref);
        vec3(m, "direction", dir);
        field(m, "scale", scale);
        if (m.get("min")) bad(GPIS_ENOTSUP, "linear mean 'min' is not supported");
        const double len = std::sqrt((double)dir[0] * dir[0] + (double)dir[1] * dir[1] + (double)dir[2] * dir[2]);
        if (!(len > 0)) bad(GPIS_EINVAL, "linear mean direction is zero");
        d->mean_kind = GPIS_MEAN_PLANE;
        double off = 0.0;
        for (int i = 0; i < 3; ++i) {
            const double n = dir[i] / len * scale;
            d->mean_params[i] = (float)n;
            off += n * ref[i];
        }
        d->mean_params[3] = (float)off;
    } else if (type == "torus") {
        float c[3] = {0, 0, 0}, R = 1.0f, r = 0.25f;
        vec3(m, "center", c);
        field(m, "major_radius", R);
        field(m, "minor_radius", r);
        d->mean_kind = GPIS_MEAN_TORUS;
        d->mean_params[0] = c[0]; d->mean_params[1] = c[1]; d->mean_params[2] = c[2];
        d->mean_params[3] = R; d->mean_params[4] = r;
    } else {
        bad(GPIS_ENOTSUP, "mean '" + type + "' is not supported");
    }
}

void gaussian_process(const Value &g, gpis_medium_desc *d)
{
    const std::string type = str(g, "type", "standard");
    if (type == "standard") {
        if (const Value *m = g.get("mean")) mean(*m, d);
        if (const Value *c = g.get("covariance")) covariance(*c, d);
        return;
    }
    if (type == "csg") {
        const Value *l = g.get("left"), *r = g.get("right");
        if (!l || !r) bad(GPIS_EINVAL, "csg needs 'left' and 'right'");
        gaussian_process(*l, d);
        if (d->mean_kind != GPIS_MEAN_TORUS) bad(GPIS_ENOTSUP, "csg supports a torus left operand");
        gpis_medium_desc rd = *d;
        gaussian_process(*r, &rd);
        if (rd.mean_kind != GPIS_MEAN_PLANE || rd.mean_params[0] != 0.0f || rd.mean_params[2] != 0.0f ||
            rd.mean_params[1] != 1.0f)
            bad(GPIS_ENOTSUP, "csg supports a linear right operand with direction (0,1,0)");
        d->mean_kind = GPIS_MEAN_TORUS_PLANE;
        d->mean_params[5] = rd.mean_params[3];
        return;
    }
    bad(GPIS_ENOTSUP, "gaussian_process '" + type + "' is not supported");
}

}  // namespace

// set by gpis_abi.cu's error channel
extern "C" int gpis_internal_set_error(int code, const char *msg);

extern "C" int gpis_medium_desc_from_json(const char *json, gpis_medium_desc *d)
{
    if (!json || !d) return gpis_internal_set_error(GPIS_EINVAL, "null argument");
    gpis_medium_desc_init(d);
    try {
        const Value v = gpis::json::parse(json);
        if (v.kind != Value::Object) bad(GPIS_EINVAL, "medium JSON must be an object");
        const std::string type = str(v, "type", "sparse_conv_noise");
        if (type != "sparse_conv_noise") bad(GPIS_ENOTSUP, "medium type '" + type + "' is not sparse_conv_noise");
        field(v, "sigma_a", d->sigma_a);
        field(v, "sigma_s", d->sigma_s);
        field(v, "density", d->density);
        d->correlation_context = context_of(str(v, "correlation_context", "goldfish"));
        const std::string im = str(v, "intersect_method", "gp_discrete");
        if (im != "gp_discrete") bad(im == "mean" ? GPIS_ENOTSUP : GPIS_EINVAL, "Invalid intersect method: '" + im + "'");
        if (const Value *g = v.get("gaussian_process")) gaussian_process(*g, d);
        field(v, "step_size", d->step_size);
        field(v, "min_step", d->min_step);
        field(v, "seed", d->seed);
        field(v, "impulse_density", d->impulse_density);
        field(v, "single_realization", d->single_realization);
        field(v, "isotropic_3D_sampling", d->isotropic_3d_sampling);
        field(v, "1D_sampling", d->one_d_sampling);
        d->sampling_scheme = scheme_of(str(v, "1D_sampling_scheme", "uni"));
        field(v, "1D_gradient_correlationXY", d->correlation_xy);
        if (const Value *s = v.get("surf_vol_phase_separate"))
            if (num(*s, "surf_vol_phase_separate") != 0.0) bad(GPIS_ENOTSUP, "surf_vol_phase_separate is not supported");
        field(v, "max_steps", d->max_steps);
        field(v, "max_bounces", d->max_bounces);
    } catch (const Err &e) {
        return gpis_internal_set_error(e.code, e.msg.c_str());
    } catch (const std::exception &e) {
        return gpis_internal_set_error(GPIS_EINVAL, e.what());
    }
    return GPIS_OK;
}
