// The compiled ionic models, keyed by the reference's ionicModel names.
#include <cstring>
#include <string>

#include "ionic_registry.h"
#include "models/alievpanfilov.cuh"
#include "models/buenoorovio.cuh"
#include "models/ord.cuh"
#include "models/tnnp.cuh"
#include "models/torord_dyncl.cuh"
#include "models/monodomainfdamanufactured.cuh"
#include "models/bidomainfdamanufactured.cuh"

#define CFG_DECLARE_MODEL(ns)                                                                  \
    extern "C" cudaError_t cfg_ionic_step_##ns##_fp64(const cfg::IonicLaunch&, int,           \
                                                      cudaStream_t, int);                     \
    extern "C" cudaError_t cfg_ionic_step_##ns##_mixed(const cfg::IonicLaunch&, int,          \
                                                       cudaStream_t, int);                    \
    extern "C" cudaError_t cfg_ionic_init_##ns##_fp64(long long, int, const unsigned char*,   \
                                                      const double*, long long, double,       \
                                                      double*, float*, double*, cudaStream_t); \
    extern "C" cudaError_t cfg_ionic_init_##ns##_mixed(long long, int, const unsigned char*,  \
                                                       const double*, long long, double,      \
                                                       double*, float*, double*,              \
                                                       cudaStream_t);                         \
    extern "C" void cfg_ionic_host_init_##ns(double*, double*, int, const double*);          \
    extern "C" cudaError_t cfg_batch_init_##ns##_fp64(const cfg::BatchLaunch&, const double*, \
                                                      int, double, cudaStream_t);             \
    extern "C" cudaError_t cfg_batch_init_##ns##_mixed(const cfg::BatchLaunch&, const double*,\
                                                       int, double, cudaStream_t);            \
    extern "C" cudaError_t cfg_batch_step_##ns##_fp64(const cfg::BatchLaunch&, int,           \
                                                      cudaStream_t);                          \
    extern "C" cudaError_t cfg_batch_step_##ns##_mixed(const cfg::BatchLaunch&, int,          \
                                                       cudaStream_t);                         \
    extern "C" cudaError_t cfg_ionic_sweep_##ns(const double*, const double*, int, int,        \
                                                const cfg::CfgStimulus&, double, double, int,  \
                                                double, int, double*, cudaStream_t);          \
    extern "C" int cfg_ionic_max_block_##ns##_fp64();                                         \
    extern "C" int cfg_ionic_max_block_##ns##_mixed();

CFG_DECLARE_MODEL(tnnp)
CFG_DECLARE_MODEL(ord)
CFG_DECLARE_MODEL(torord_dyncl)
CFG_DECLARE_MODEL(alievpanfilov)
CFG_DECLARE_MODEL(buenoorovio)
CFG_DECLARE_MODEL(monodomainfdamanufactured)
CFG_DECLARE_MODEL(bidomainfdamanufactured)

namespace cfg {
namespace {

template <class M>
struct Tables {
    int wide[2][M::NS];
    int slot[2][M::NS];
    Tables()
    {
        for (int i = 0; i < M::NS; ++i) {
            wide[0][i] = 1;
            slot[0][i] = Layout<M, true>::slot(i);
            wide[1][i] = int((M::WIDE_MASK >> i) & 1ull);
            slot[1][i] = Layout<M, false>::slot(i);
        }
    }
};

#define CFG_STEP_FN(NSP, prec, sv)                                                               \
    [](const IonicLaunch& p, cudaStream_t s, int b) {                                           \
        return cfg_ionic_step_##NSP##_##prec(p, sv, s, b);                                       \
    }

#define CFG_MODEL_ENTRY(KEY, NSP)                                                                \
    [] {                                                                                        \
        static Tables<NSP::Model> t;                                                             \
        IonicModelOps o{};                                                                      \
        o.name = KEY;                                                                           \
        o.ns = NSP::NS;                                                                          \
        o.nc = NSP::NC;                                                                          \
        o.n_wide[0] = Layout<NSP::Model, true>::n_wide();                                        \
        o.n_wide[1] = Layout<NSP::Model, false>::n_wide();                                       \
        o.wide_of = &t.wide[0][0];                                                              \
        o.slot_of = &t.slot[0][0];                                                              \
        o.state_names = NSP::STATE_NAMES;                                                        \
        o.tissues = NSP::TISSUES;                                                                \
        o.iion_scale = NSP::IION_SCALE;                                                          \
        o.time_scale = NSP::TIME_SCALE;                                                          \
        o.vm_map = NSP::VM_MAP;                                                                  \
        o.step[0][0] = CFG_STEP_FN(NSP, fp64, 0);                                                \
        o.step[0][1] = CFG_STEP_FN(NSP, fp64, 1);                                                \
        o.step[1][0] = CFG_STEP_FN(NSP, mixed, 0);                                               \
        o.step[1][1] = CFG_STEP_FN(NSP, mixed, 1);                                               \
        o.init[0] = cfg_ionic_init_##NSP##_fp64;                                                 \
        o.init[1] = cfg_ionic_init_##NSP##_mixed;                                                \
        o.host_init = cfg_ionic_host_init_##NSP;                                                 \
        o.batch_init[0] = cfg_batch_init_##NSP##_fp64;                                           \
        o.batch_init[1] = cfg_batch_init_##NSP##_mixed;                                          \
        o.batch_step[0] = cfg_batch_step_##NSP##_fp64;                                           \
        o.batch_step[1] = cfg_batch_step_##NSP##_mixed;                                          \
        o.nsd = NSP::NSD;                                                                        \
        o.ca_state = NSP::CA_STATE;                                                              \
        o.na = NSP::NA;                                                                          \
        o.state_strings = NSP::STATE_STRINGS;                                                    \
        o.alg_strings = NSP::ALG_STRINGS;                                                        \
        o.sweep_currents = NSP::SWEEP_CURRENTS;                                                  \
        o.sweep_deps = NSP::SWEEP_DEPS;                                                          \
        o.sweep = cfg_ionic_sweep_##NSP;                                                         \
        o.max_block[0] = cfg_ionic_max_block_##NSP##_fp64;                                       \
        o.max_block[1] = cfg_ionic_max_block_##NSP##_mixed;                                      \
        return o;                                                                               \
    }()

const IonicModelOps* table()
{
    static const IonicModelOps models[] = {
        CFG_MODEL_ENTRY("TNNP", tnnp),
        CFG_MODEL_ENTRY("ORd", ord),
        CFG_MODEL_ENTRY("ToRORd_dynCl", torord_dyncl),
        CFG_MODEL_ENTRY("AlievPanfilov", alievpanfilov),
        CFG_MODEL_ENTRY("BuenoOrovio", buenoorovio),
        CFG_MODEL_ENTRY("monodomainFDAManufactured", monodomainfdamanufactured),
        CFG_MODEL_ENTRY("bidomainFDAManufactured", bidomainfdamanufactured),
        IonicModelOps{},
    };
    return models;
}

}  // namespace

const IonicModelOps* find_ionic_model(const char* name)
{
    if (!name) return nullptr;
    for (const IonicModelOps* m = table(); m->name; ++m)
        if (std::strcmp(m->name, name) == 0) return m;
    return nullptr;
}

const char* ionic_model_names()
{
    static std::string s = [] {
        std::string r;
        for (const IonicModelOps* m = table(); m->name; ++m) {
            if (!r.empty()) r += ' ';
            r += m->name;
        }
        return r;
    }();
    return s.c_str();
}

}  // namespace cfg
