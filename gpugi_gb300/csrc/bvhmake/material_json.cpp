// Material records from gpugi's scene JSON ("materials": {name: {...}}), the
// file bvhmake writes next to a scene (bvhmake/main.cpp:105-117) and
// Scene::LoadMaterial reads (gpugi/scene/scene.cpp:132-180). A small JSON
// reader (objects, arrays, numbers, strings, true/false/null) and the
// parameter mapping of LoadMaterial with its defaults:
//   refractionIndex 1.5, specularColor (fresnel0) 0.03, fresnel1 = 1 - fresnel0,
//   roughness 1 -> Phong exponent 1 / (roughness^2 + 1e-20), albedo 0.5,
//   opacity 1, reflectiveness (1, 1, 1, exponent), emissivity 0.
// Textures are not supported: a string value is rejected.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../../include/gpugi_bvhmake.h"

namespace {

struct JValue {
    enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
    double num = 0.0;
    std::string str;
    std::vector<JValue> arr;
    std::vector<std::pair<std::string, JValue>> obj;
    const JValue* get(const std::string& k) const {
        for (const auto& kv : obj)
            if (kv.first == k) return &kv.second;
        return nullptr;
    }
};

struct Parser {
    const char* p;
    const char* end;
    std::string err;
    int depth = 0;
    void ws() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
    }
    bool fail(const char* m) {
        if (err.empty()) err = m;
        return false;
    }
    bool str(std::string& out) {
        if (p >= end || *p != '"') return fail("expected a string");
        ++p;
        while (p < end && *p != '"') {
            if (*p == '\\') {
                if (++p >= end) break;
                const char c = *p++;
                switch (c) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'u':  // keep the escape verbatim (names are ASCII in practice)
                        out += "\\u";
                        break;
                    default: out += c;
                }
            } else {
                out += *p++;
            }
        }
        if (p >= end) return fail("unterminated string");
        ++p;
        return true;
    }
    bool value(JValue& v) {
        if (++depth > 64) return fail("nesting too deep");
        ws();
        if (p >= end) return fail("unexpected end");
        bool ok = true;
        if (*p == '{') {
            v.kind = JValue::OBJ;
            ++p;
            ws();
            if (p < end && *p == '}') {
                ++p;
            } else {
                while (ok) {
                    ws();
                    std::string k;
                    if (!(ok = str(k))) break;
                    ws();
                    if (p >= end || *p != ':') { ok = fail("expected ':'"); break; }
                    ++p;
                    JValue child;
                    if (!(ok = value(child))) break;
                    v.obj.emplace_back(std::move(k), std::move(child));
                    ws();
                    if (p < end && *p == ',') { ++p; continue; }
                    if (p < end && *p == '}') { ++p; break; }
                    ok = fail("expected ',' or '}'");
                }
            }
        } else if (*p == '[') {
            v.kind = JValue::ARR;
            ++p;
            ws();
            if (p < end && *p == ']') {
                ++p;
            } else {
                while (ok) {
                    JValue child;
                    if (!(ok = value(child))) break;
                    v.arr.push_back(std::move(child));
                    ws();
                    if (p < end && *p == ',') { ++p; continue; }
                    if (p < end && *p == ']') { ++p; break; }
                    ok = fail("expected ',' or ']'");
                }
            }
        } else if (*p == '"') {
            v.kind = JValue::STR;
            ok = str(v.str);
        } else if (end - p >= 4 && std::strncmp(p, "true", 4) == 0) {
            v.kind = JValue::BOOL, v.num = 1.0, p += 4;
        } else if (end - p >= 5 && std::strncmp(p, "false", 5) == 0) {
            v.kind = JValue::BOOL, v.num = 0.0, p += 5;
        } else if (end - p >= 4 && std::strncmp(p, "null", 4) == 0) {
            v.kind = JValue::NUL, p += 4;
        } else {
            std::string tok;
            while (p < end && (std::strchr("+-.eE0123456789", *p) != nullptr)) tok += *p++;
            if (tok.empty()) return fail("unexpected character");
            char* e = nullptr;
            v.kind = JValue::NUM;
            v.num = std::strtod(tok.c_str(), &e);
            if (!e || *e) ok = fail("bad number");
        }
        --depth;
        return ok;
    }
};

thread_local std::string g_jsonError;

// Value of a parameter as n floats: a number or an array of numbers; a
// shorter array repeats its last element (bim's scalar reads of 1-element
// arrays). Returns false if absent; sets *bad for a string (texture).
bool numbers(const JValue* v, float* out, int n, bool* bad) {
    if (!v) return false;
    if (v->kind == JValue::NUM) {
        for (int i = 0; i < n; ++i) out[i] = (float)v->num;
        return true;
    }
    if (v->kind == JValue::ARR && !v->arr.empty()) {
        for (int i = 0; i < n; ++i) {
            const JValue& e = v->arr[(size_t)i < v->arr.size() ? (size_t)i : v->arr.size() - 1];
            if (e.kind != JValue::NUM) {
                *bad = true;
                return false;
            }
            out[i] = (float)e.num;
        }
        return true;
    }
    *bad = true;
    return false;
}

}  // namespace

extern "C" {

int gpugi_materials_from_json(const char* json, const char* const* names, uint32_t numNames, float* records) {
    if (!json || (numNames && (!names || !records))) return -1;
    Parser ps{json, json + std::strlen(json)};
    JValue root;
    if (!ps.value(root) || root.kind != JValue::OBJ) {
        g_jsonError = "JSON: " + (ps.err.empty() ? std::string("root is not an object") : ps.err);
        return -2;
    }
    const JValue* mats = root.get("materials");
    if (!mats || mats->kind != JValue::OBJ) {
        g_jsonError = "JSON has no \"materials\" object";
        return -3;
    }
    for (uint32_t m = 0; m < numNames; ++m) {
        float* r = records + 24 * (size_t)m;
        const JValue* mat = mats->get(names[m] ? names[m] : "");
        if (!mat || mat->kind != JValue::OBJ) {
            g_jsonError = std::string("material not found: ") + (names[m] ? names[m] : "(null)");
            return -4;
        }
        bool bad = false;
        float ior = 1.5f, f0[3] = {0.03f, 0.03f, 0.03f}, rough = 1.0f, albedo[3] = {0.5f, 0.5f, 0.5f}, opacity = 1.0f,
              emis[3] = {0.0f, 0.0f, 0.0f};
        numbers(mat->get("refractionIndex"), &ior, 1, &bad);
        numbers(mat->get("specularColor"), f0, 3, &bad);
        numbers(mat->get("roughness"), &rough, 1, &bad);
        numbers(mat->get("albedo"), albedo, 3, &bad);
        numbers(mat->get("opacity"), &opacity, 1, &bad);
        numbers(mat->get("emissivity"), emis, 3, &bad);
        const float exponent = 1.0f / (rough * rough + 1e-20f);
        float refl[4] = {1.0f, 1.0f, 1.0f, exponent};
        const JValue* rv = mat->get("reflectiveness");
        if (rv && rv->kind == JValue::ARR && rv->arr.size() >= 4) numbers(rv, refl, 4, &bad);
        else numbers(rv, refl, 3, &bad);
        if (bad) {
            g_jsonError = std::string("material ") + names[m] + ": textures and non-numeric values are not supported";
            return -5;
        }
        // gpugi_material layout: diffuse, ior | opacity, pad | reflectiveness | emissivity, pad | fresnel0, pad | fresnel1, pad
        std::memset(r, 0, 24 * sizeof(float));
        for (int i = 0; i < 3; ++i) {
            r[i] = albedo[i];
            r[4 + i] = opacity;
            r[12 + i] = emis[i];
            r[16 + i] = f0[i];
            r[20 + i] = 1.0f - f0[i];
        }
        r[3] = ior;
        for (int i = 0; i < 4; ++i) r[8 + i] = refl[i];
    }
    return 0;
}

const char* gpugi_materials_json_error(void) { return g_jsonError.c_str(); }

}  // extern "C"
