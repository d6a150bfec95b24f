/* disney.cuh - the Disney principled BSDF of the OptiX 7 and PrimeAdaptive cores (their default kernels/bsdf.h
 * branch): lib/sharedBSDFs/disney.h (diffuse with Hanrahan-Krueger subsurface, sheen, GGX specular, GTR1
 * clearcoat, component sampling by luminance-weighted cdf), ggxmdf.h (anisotropic GGX and GTR1 distributions,
 * visible-normal sampling) and frosted.h (rough dielectric reflection / refraction), adapted there from AppleSeed.
 *
 * Operation order is the reference's, with its CUDA branches (sincosf in the samplers) and the core's own
 * transcendentals (sincos_cw, exp_cw, log_at, pow_at) and normalize (v * (1 / sqrt(dot))). Values the reference
 * leaves unset on measure-zero paths are zero here: the component pdf and the running contribution when a sampled
 * or evaluated direction lies exactly in the tangent plane. */
#pragma once
#include "shading.cuh"

namespace lh2g {
namespace disney {

/* the material parameters (tools_shared.h:40-54 CHAR2FLT layout) */
LH2G_DEV float METALLIC(const Shading& s) { return char2flt(s.params[0], 0); }
LH2G_DEV float SUBSURFACE(const Shading& s) { return char2flt(s.params[0], 8); }
LH2G_DEV float SPECULAR(const Shading& s) { return char2flt(s.params[0], 16); }
LH2G_DEV float SPECTINT(const Shading& s) { return char2flt(s.params[1], 0); }
LH2G_DEV float ANISOTROPIC(const Shading& s) { return char2flt(s.params[1], 8); }
LH2G_DEV float SHEEN(const Shading& s) { return char2flt(s.params[1], 16); }
LH2G_DEV float SHEENTINT(const Shading& s) { return char2flt(s.params[1], 24); }
LH2G_DEV float CLEARCOAT(const Shading& s) { return char2flt(s.params[2], 0); }
LH2G_DEV float CLEARCOATGLOSS(const Shading& s) { return char2flt(s.params[2], 8); }
LH2G_DEV float3 TINT(const Shading& s) { return make_float3(s.tint.x, s.tint.y, s.tint.z); }
LH2G_DEV float LUMINANCE(const Shading& s) { return s.tint.w; }

LH2G_DEV float sqr(float x) { return x * x; }
LH2G_DEV float saturate(float x) { return fmaxf(0.0f, fminf(1.0f, x)); }
LH2G_DEV float lerp(float a, float b, float t) { return a + t * (b - a); }
LH2G_DEV float mix(float a, float b, float x) { return x <= 0 ? a : x >= 1 ? b : lerp(a, b, x); }
LH2G_DEV float clampf(float f, float a, float b) { return fmaxf(a, fminf(f, b)); }
LH2G_DEV float3 world2tangent(const float3 V, const float3 N, const float3 T, const float3 B) { return make_float3(dot(V, T), dot(V, B), dot(V, N)); }
LH2G_DEV float3 tangent2world(const float3 V, const float3 N, const float3 T, const float3 B) { return V.x * T + V.y * B + V.z * N; }
/* common_functions.h DiffuseReflectionCosWeighted with a tangent frame */
LH2G_DEV float3 cosine_sample(const float r0, const float r1, const float3 N, const float3 T, const float3 B) {
    const float term1 = TWOPI * r0, term2 = sqrtf(1 - r1);
    float s, c;
    sincos_cw(term1, &s, &c);
    return (c * term2 * T) + (s * term2) * B + sqrtf(r1) * N;
}

/* ---- ggxmdf.h ---- */
LH2G_DEV float ggx_D(const float3 m, const float ax, const float ay) {
    if (m.z == 0) return sqr(ax) * INVPI;
    const float c2 = sqr(m.z), sinT = sqrtf(fmaxf(0.0f, 1 - c2)), tan2 = (1.0f - c2) / c2;
    const float stretched = (ax == ay || sinT == 0.0f) ? 1.0f / sqr(ax) : sqr(m.x / (sinT * ax)) + sqr(m.y / (sinT * ay));
    return 1.0f / (PI * ax * ay * sqr(c2) * sqr(1.0f + tan2 * stretched));
}
LH2G_DEV float ggx_lambda(const float3 v, const float ax, const float ay) {
    if (v.z == 0) return 0;
    const float c2 = v.z * v.z, sinT = sqrtf(fmaxf(0.0f, 1 - c2));
    const float proj = (ax == ay || sinT == 0.0f) ? ax : sqrtf(sqr((v.x * ax) / sinT) + sqr((v.y * ay) / sinT));
    const float tan2 = sqr(sinT) / c2, a2rcp = sqr(proj) * tan2;
    return (-1.0f + sqrtf(1.0f + a2rcp)) * 0.5f;
}
LH2G_DEV float ggx_G(const float3 wi, const float3 wo, const float ax, const float ay) { return 1.0f / (1.0f + ggx_lambda(wo, ax, ay) + ggx_lambda(wi, ax, ay)); }
LH2G_DEV float ggx_G1(const float3 v, const float ax, const float ay) { return 1.0f / (1.0f + ggx_lambda(v, ax, ay)); }
/* visible-normal sampling (ggxmdf.h GGXMDF_sample, the CUDA branch) */
LH2G_DEV float3 ggx_sample(const float3 v, const float r0, const float r1, const float ax, const float ay) {
    const float sgn = v.z < 0.0f ? -1.0f : 1.0f;
    const float3 st = normalize(make_float3(sgn * v.x * ax, sgn * v.y * ay, sgn * v.z));
    const float3 t1 = v.z < 0.9999f ? normalize(cross(st, make_float3(0, 0, 1))) : make_float3(1, 0, 0);
    const float3 t2 = cross(t1, st);
    const float a = 1.0f / (1.0f + st.z), r = sqrtf(r0);
    const float phi = r1 < a ? (r1 / a * PI) : (PI + (r1 - a) / (1.0f - a) * PI);
    float p1, p2;
    sincos_cw(phi, &p2, &p1);
    p1 *= r;
    p2 *= r * (r1 < a ? 1.0f : st.z);
    const float3 h = p1 * t1 + p2 * t2 + sqrtf(fmaxf(0.0f, 1.0f - p1 * p1 - p2 * p2)) * st;
    return normalize(make_float3(h.x * ax, h.y * ay, fmaxf(0.0f, h.z)));
}
LH2G_DEV float ggx_pdf(const float3 v, const float3 m, const float ax, const float ay) {
    if (v.z == 0.0f) return 0;
    return ggx_G1(v, ax, ay) * fabsf(dot(v, m)) * ggx_D(m, ax, ay) / fabsf(v.z);
}
LH2G_DEV float gtr1_D(const float3 m, const float ax) {
    const float alpha = clampf(ax, 0.001f, 0.999f), a2 = sqr(alpha);
    const float a = (a2 - 1.0f) / (PI * log_at(a2)), b = (1 / (1 + (a2 - 1) * sqr(m.z)));
    return a * b;
}
LH2G_DEV float gtr1_lambda(const float3 v, const float ax) {
    if (v.z == 0) return 0;
    const float c2 = sqr(v.z), sinT = sqrtf(fmaxf(0.0f, 1.0f - c2));
    if (sinT == 0) return 0;
    const float cot2 = c2 / sqr(sinT), cot = sqrtf(cot2), alpha2 = sqr(clampf(ax, 0.001f, 0.999f));
    const float a = sqrtf(cot2 + alpha2), b = sqrtf(cot2 + 1.0f), c = log_at(cot + b), d = log_at(cot + a);
    return (a - b + cot * (c - d)) / (cot * log_at(alpha2));
}
LH2G_DEV float gtr1_G(const float3 wi, const float3 wo, const float ax) { return 1.0f / (1.0f + gtr1_lambda(wo, ax) + gtr1_lambda(wi, ax)); }
LH2G_DEV float3 gtr1_sample(const float r0, const float r1, const float ax) {
    const float alpha = clampf(ax, 0.001f, 0.999f), a2 = sqr(alpha);
    const float c2 = (1.0f - pow_at(a2, 1.0f - r0)) / (1.0f - a2), sinT = sqrtf(fmaxf(0.0f, 1.0f - c2));
    float sp, cp;
    sincos_cw(TWOPI * r1, &sp, &cp);
    return make_float3(cp * sinT, sp * sinT, sqrtf(c2));
}
LH2G_DEV float gtr1_pdf(const float3 m, const float ax) { return gtr1_D(m, ax) * fabsf(m.z); }
LH2G_DEV void alpha_from_roughness(const float roughness, const float anisotropy, float& ax, float& ay) {
    const float sq = roughness * roughness, aspect = sqrtf(1.0f + anisotropy * (anisotropy < 0 ? 0.9f : -0.9f));
    ax = fmaxf(0.001f, sq / aspect), ay = fmaxf(0.001f, sq * aspect);
}

/* ---- frosted.h (rough dielectric) ---- */
LH2G_DEV float fresnel_dielectric(const float eta, const float ci, const float ct) {
    if (ci == 0 && ct == 0) return 1;
    const float k0 = eta * ct, k1 = eta * ci;
    return 0.5f * (sqr((ci - k0) / (ci + k0)) + sqr((ct - k1) / (ct + k1)));
}
LH2G_DEV float fresnel_reflectance(const float ci, const float eta, float& ct) {
    const float st2 = (1 - sqr(ci)) * sqr(eta);
    if (st2 > 1) { ct = 0; return 1; }
    ct = fminf(sqrtf(fmaxf(1 - st2, 0.0f)), 1.0f);
    return fresnel_dielectric(eta, fabsf(ci), ct);
}
LH2G_DEV float3 refracted_direction(const float3 wo, const float3 m, const float cwm, const float ct, const float rcpEta) {
    const float3 wi = cwm > 0 ? (rcpEta * cwm - ct) * m - rcpEta * wo : (rcpEta * cwm + ct) * m - rcpEta * wo;
    return wi * ((3 - dot(wi, wi)) * 0.5f);
}
LH2G_DEV float choose_reflection(const float F) {
    const float r = F * 1, t = (1 - F) * 1, sum = r + t;
    return sum != 0 ? r / sum : 1;
}
LH2G_DEV float3 half_reflection(const float3 wo, const float3 wi) {
    const float3 h = normalize(wi + wo);
    return h.z < 0 ? (h * -1) : h;
}
LH2G_DEV float3 half_refraction(const float3 wo, const float3 wi, const float eta) {
    const float3 h = normalize(wo + eta * wi);
    return h.z < 0 ? (h * -1) : h;
}
LH2G_DEV float3 eval_reflection(const float3 color, const float3 wo, const float3 wi, const float3 m, const float ax, const float ay, const float F) {
    const float denom = fabsf(4 * wo.z * wi.z);
    if (denom == 0) return mk3(0);
    const float D = ggx_D(m, ax, ay), G = ggx_G(wi, wo, ax, ay);
    return color * (F * D * G / denom);
}
LH2G_DEV float3 eval_refraction(const float eta, const float3 color, const float3 wo, const float3 wi, const float3 m, const float ax, const float ay,
                                const float Tr) {
    if (wo.z == 0 || wi.z == 0) return mk3(0);
    const float cih = dot(m, wi), coh = dot(m, wo), dots = (cih * coh) / (wi.z * wo.z), sd = coh + eta * cih;
    if (fabsf(sd) < 1.0e-6f) return mk3(0);
    const float D = ggx_D(m, ax, ay), G = ggx_G(wi, wo, ax, ay);
    float mult = fabsf(dots) * Tr * D * G / sqr(sd);
    mult *= sqr(eta);   /* not adjoint */
    return color * mult;
}
LH2G_DEV float reflection_jacobian(const float coh) { return coh == 0 ? 0.0f : 1 / (4 * fabsf(coh)); }
LH2G_DEV float refraction_jacobian(const float3 wo, const float3 wi, const float3 m, const float eta) {
    const float cih = dot(m, wi), coh = dot(m, wo), sd = coh + eta * cih;
    if (fabsf(sd) < 1.0e-6f) return 0;
    return fabsf(cih) * sqr(eta / sd);
}

/* ---- disney.h ---- */
LH2G_DEV float schlick(const float u) { const float m = saturate(1.0f - u), m2 = sqr(m), m4 = sqr(m2); return m4 * m; }
LH2G_DEV float clearcoat_roughness(const Shading& s) { return mix(0.1f, 0.001f, CLEARCOATGLOSS(s)); }
LH2G_DEV float3 specular_fresnel(const Shading& s, const float3 o, const float3 h) {
    const float st = SPECTINT(s), M = METALLIC(s);
    float3 v = (1.0f - st) + st * TINT(s);   /* mix_one_with_spectra */
    v = v * (SPECULAR(s) * 0.08f);
    v = (1.0f - M) * v + M * s.color;        /* mix_spectra */
    const float f = schlick(fabsf(dot(o, h)));
    return (1.0f - f) * v + f;               /* mix_spectra_with_one */
}
LH2G_DEV float3 clearcoat_fresnel(const Shading& s, const float3 o, const float3 h) {
    return mk3(mix(0.04f, 1.0f, schlick(fabsf(dot(o, h)))) * 0.25f * CLEARCOAT(s));
}

/* sample_mf<GGXMDF / GTR1MDF> (disney.h): pdf and value are left as they are on the early exits */
template <bool GTR1>
LH2G_DEV void sample_mf(const Shading& s, const float r0, const float r1, const float ax, const float ay, const float3 wol, float3& wil, float& pdf, float3& value) {
    if (wol.z == 0) { value = mk3(0); pdf = 0; return; }
    const float3 m = GTR1 ? gtr1_sample(r0, r1, ax) : ggx_sample(wol, r0, r1, ax, ay);
    wil = reflect(wol * -1.0f, m);
    if (wil.z == 0) return;
    const float coh = dot(wol, m);
    pdf = (GTR1 ? gtr1_pdf(m, ax) : ggx_pdf(wol, m, ax, ay)) / fabsf(4.0f * coh);
    if (pdf < 1.0e-6f) return;
    const float D = GTR1 ? gtr1_D(m, ax) : ggx_D(m, ax, ay);
    const float G = GTR1 ? gtr1_G(wil, wol, ax) : ggx_G(wil, wol, ax, ay);
    value = GTR1 ? clearcoat_fresnel(s, wol, m) : specular_fresnel(s, wol, m);
    value = value * (D * G);
}
/* evaluate_mf: bsdf is left as it is on the early exits */
template <bool GTR1>
LH2G_DEV float evaluate_mf(const Shading& s, const float ax, const float ay, const float3 wol, const float3 wil, const float3 m, float3& bsdf) {
    if (wol.z == 0 || wil.z == 0) return 0;
    const float coh = dot(wol, m);
    if (coh == 0) return 0;
    const float D = GTR1 ? gtr1_D(m, ax) : ggx_D(m, ax, ay);
    const float G = GTR1 ? gtr1_G(wil, wol, ax) : ggx_G(wil, wol, ax, ay);
    bsdf = GTR1 ? clearcoat_fresnel(s, wol, m) : specular_fresnel(s, wol, m);
    bsdf = bsdf * (D * G / fabsf(4.0f * wol.z * wil.z));
    return (GTR1 ? gtr1_pdf(m, ax) : ggx_pdf(wol, m, ax, ay)) / fabsf(4.0f * coh);
}
LH2G_DEV float evaluate_diffuse(const Shading& s, const float3 iN, const float3 wow, const float3 wiw, const float3 m, float3& value) {
    const float con = dot(iN, wow), cin = dot(iN, wiw), cih = dot(wiw, m);
    const float fl = schlick(cin), fv = schlick(con), R = ROUGHNESS(s), SS = SUBSURFACE(s);
    float fd = 0;
    if (SS != 1.0f) {
        const float fd90 = 0.5f + 2.0f * sqr(cih) * R;
        fd = mix(1.0f, fd90, fl) * mix(1.0f, fd90, fv);
    }
    if (SS > 0) {
        const float fss90 = sqr(cih) * R, fss = mix(1.0f, fss90, fl) * mix(1.0f, fss90, fv);
        const float ss = 1.25f * (fss * (1.0f / (fabsf(con) + fabsf(cin)) - 0.5f) + 0.5f);
        fd = mix(fd, ss, SS);
    }
    value = s.color * fd * INVPI * (1.0f - METALLIC(s));
    return fabsf(cin) * INVPI;
}
LH2G_DEV float evaluate_sheen(const Shading& s, const float3 wiw, const float3 m, float3& value) {
    const float fh = schlick(dot(wiw, m)), st = SHEENTINT(s);
    value = (1.0f - st) + st * TINT(s);
    value = value * (fh * SHEEN(s) * (1.0f - METALLIC(s)));
    return 1.0f / (2 * PI);
}
/* the component weights (luminance-weighted diffuse, sheen, specular, clearcoat), normalised */
LH2G_DEV float4 weights_of(const Shading& s) {
    const float M = METALLIC(s);
    float4 w = make_float4(lerp(LUMINANCE(s), 0, M), lerp(SHEEN(s), 0, M), lerp(SPECULAR(s), 1, M), CLEARCOAT(s) * 0.25f);
    w = w * (1.0f / (w.x + w.y + w.z + w.w));
    return w;
}

/* SampleBSDF (disney.h) with the shading frame and r0..r2; pdf and wiw are left as they are where the reference
 * leaves them */
LH2G_DEV float3 SampleBSDF(const Shading& s, float3 iN, const float3 N, const float3 iT, const float3 wow, const float distance, const float r0,
                           const float r1, const float r2, float3& wiw, float& pdf, bool& specular) {
    const float flip = (dot(wow, N) < 0) ? -1 : 1;
    iN = iN * flip;
    const float3 B = normalize(cross(iN, iT)), T = normalize(cross(iN, B));
    const float TR = TRANSMISSION(s);
    if (r0 < TR) {
        specular = true;
        const float r3 = r0 / TR;
        const float3 wol = world2tangent(wow, iN, T, B);
        const float eta = flip < 0 ? (1 / ETA(s)) : ETA(s);
        if (eta == 1) return mk3(0);
        const float3 beer = make_float3(exp_cw(-s.transmittance.x * distance * 2.0f), exp_cw(-s.transmittance.y * distance * 2.0f),
                                        exp_cw(-s.transmittance.z * distance * 2.0f));
        float ax, ay;
        alpha_from_roughness(ROUGHNESS(s), ANISOTROPIC(s), ax, ay);
        const float3 m = ggx_sample(wol, r1, r3, ax, ay);
        const float rcpEta = 1 / eta, cwm = clampf(dot(wol, m), -1.0f, 1.0f);
        float ct, jac;
        const float F = fresnel_reflectance(cwm, eta, ct);
        float3 wil, ret;
        if (r2 < F) {
            wil = reflect(wol * -1.0f, m);
            if (wil.z * wol.z <= 0) return mk3(0);
            ret = eval_reflection(s.color, wol, wil, m, ax, ay, F);
            pdf = F, jac = reflection_jacobian(cwm);
        } else {
            wil = refracted_direction(wol, m, cwm, ct, eta);
            if (wil.z * wol.z > 0) return mk3(0);
            ret = eval_refraction(rcpEta, s.color, wol, wil, m, ax, ay, 1 - F);
            pdf = 1 - F, jac = refraction_jacobian(wol, wil, m, rcpEta);
        }
        pdf *= jac * ggx_pdf(wol, m, ax, ay);
        if (pdf > 1.0e-6f) wiw = tangent2world(wil, iN, T, B);
        return ret * beer;
    }
    const float r3 = (r0 - TR) / (1 - TR);
    float4 w = weights_of(s);
    const float4 cdf = make_float4(w.x, w.x + w.y, w.x + w.y + w.z, 0);
    float probability, cpdf = 0;
    float3 contrib = mk3(0), value = mk3(0);
    if (r3 < cdf.y) {
        const float r2b = r3 / cdf.y;
        wiw = cosine_sample(r2b, r1, iN, T, B);
        const float3 m = normalize(wiw + wow);
        if (r3 < cdf.x) {
            cpdf = evaluate_diffuse(s, iN, wow, wiw, m, value);
            probability = w.x * cpdf, w.x = 0;
        } else {
            cpdf = evaluate_sheen(s, wiw, m, value);
            probability = w.y * cpdf, w.y = 0;
        }
    } else {
        const float3 wol = world2tangent(wow, iN, T, B);
        float3 wil = mk3(0);
        if (r3 < cdf.z) {
            const float r2b = (r3 - cdf.y) / (cdf.z - cdf.y);
            float ax, ay;
            alpha_from_roughness(ROUGHNESS(s), ANISOTROPIC(s), ax, ay);
            sample_mf<false>(s, r2b, r1, ax, ay, wol, wil, cpdf, value);
            probability = w.z * cpdf, w.z = 0;
        } else {
            const float r2b = (r3 - cdf.z) / (1 - cdf.z);
            const float a = clearcoat_roughness(s);
            sample_mf<true>(s, r2b, r1, a, a, wol, wil, cpdf, value);
            probability = w.w * cpdf, w.w = 0;
        }
        value = value * (1.0f / fabsf(4.0f * wol.z * wil.z));
        wiw = tangent2world(wil, iN, T, B);
    }
    if (w.x + w.y > 0) {
        const float3 m = normalize(wiw + wow);
        if (w.x > 0) probability += w.x * evaluate_diffuse(s, iN, wow, wiw, m, contrib), value = value + contrib;
        if (w.y > 0) probability += w.y * evaluate_sheen(s, wiw, m, contrib), value = value + contrib;
    }
    if (w.z + w.w > 0) {
        const float3 wol = world2tangent(wow, iN, T, B), wil = world2tangent(wiw, iN, T, B), m = normalize(wol + wil);
        if (w.z > 0) {
            float ax, ay;
            alpha_from_roughness(ROUGHNESS(s), ANISOTROPIC(s), ax, ay);
            probability += w.z * evaluate_mf<false>(s, ax, ay, wol, wil, m, contrib);
            value = value + contrib;
        }
        if (w.w > 0) {
            const float a = clearcoat_roughness(s);
            probability += w.w * evaluate_mf<true>(s, a, a, wol, wil, m, contrib);
            value = value + contrib;
        }
    }
    pdf = probability > 1.0e-6f ? probability : 0;
    return value;
}

/* EvaluateBSDF (disney.h) */
LH2G_DEV float3 EvaluateBSDF(const Shading& s, const float3 iN, const float3 iT, const float3 wow, const float3 wiw, float& pdf) {
    if (TRANSMISSION(s) > 0.5f) {
        const float3 B = normalize(cross(iN, iT)), T = normalize(cross(iN, B));
        const float3 wol = world2tangent(wow, iN, T, B), wil = world2tangent(wiw, iN, T, B);
        const float eta = wol.z > 0 ? ETA(s) : (1.0f / ETA(s));
        if (eta == 1) { pdf = 0; return mk3(0); }
        float ax, ay, jac;
        alpha_from_roughness(ROUGHNESS(s), ANISOTROPIC(s), ax, ay);
        float3 ret, m;
        if (wil.z * wol.z >= 0) {
            m = half_reflection(wol, wil);
            const float cwm = dot(wol, m);
            float ct;
            const float F = fresnel_reflectance(cwm, 1 / eta, ct);
            ret = eval_reflection(s.color, wol, wil, m, ax, ay, F);
            pdf = choose_reflection(F), jac = reflection_jacobian(cwm);
        } else {
            m = half_refraction(wol, wil, eta);
            const float cwm = dot(wol, m);
            float ct;
            const float F = fresnel_reflectance(cwm, 1 / eta, ct);
            ret = eval_refraction(eta, s.color, wol, wil, m, ax, ay, 1 - F);
            pdf = 1 - choose_reflection(F), jac = refraction_jacobian(wol, wil, m, eta);
        }
        pdf *= jac * ggx_pdf(wol, m, ax, ay);
        return ret;
    }
    if (ROUGHNESS(s) <= 0.001f) { pdf = 0; return mk3(0); }
    const float3 B = normalize(cross(iN, iT)), T = normalize(cross(iN, B));
    const float4 w = weights_of(s);
    pdf = 0;
    float3 value = mk3(0);
    if (w.x + w.y > 0) {
        const float3 m = normalize(wiw + wow);
        if (w.x > 0) pdf += w.x * evaluate_diffuse(s, iN, wow, wiw, m, value);
        if (w.y > 0) pdf += w.y * evaluate_sheen(s, wiw, m, value);   /* overwrites the diffuse value, as the reference does */
    }
    if (w.z + w.w > 0) {
        const float3 wol = world2tangent(wow, iN, T, B), wil = world2tangent(wiw, iN, T, B), m = normalize(wol + wil);
        if (w.z > 0) {
            float ax, ay;
            alpha_from_roughness(ROUGHNESS(s), ANISOTROPIC(s), ax, ay);
            float3 c = mk3(0);
            const float sp = evaluate_mf<false>(s, ax, ay, wol, wil, m, c);
            if (sp > 0) pdf += w.z * sp, value = value + c;
        }
        if (w.w > 0) {
            const float a = clearcoat_roughness(s);
            float3 c = mk3(0);
            const float cp = evaluate_mf<true>(s, a, a, wol, wil, m, c);
            if (cp > 0) pdf += w.w * cp, value = value + c;
        }
    }
    return value;
}

}  // namespace disney
}  // namespace lh2g
