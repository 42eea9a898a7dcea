/* CPU oracle for the monodomain time step - TEST INFRASTRUCTURE ONLY.
 *
 * Nothing in the product links this code.  It is imported by tests/, by the
 * smoke check and by bench.py's CPU-baseline leg, always as the checker.
 *
 * Shared helpers for the generated model files in oracle/models/.
 */
#ifndef ORACLE_COMMON_H
#define ORACLE_COMMON_H

#include <math.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Single-cell S1/S2 protocol; fields as in StimulusProtocol
 * (src/genericWriter/stimulusIO.H:32-53). */
typedef struct oracle_stimulus {
    double start;
    double period_s1;
    double duration;
    double amplitude;
    int n1;
    double period_s2;
    int n2;
} oracle_stimulus;

/* stimulusIO::computeStimulus (src/genericWriter/stimulusIO.C:238-286):
 * S1 train, then an S2 train starting where S1 ends; both ends inclusive. */
static inline double oracle_stimulus_current(double t, const oracle_stimulus* s)
{
    double istim = 0.0;
    if (!s) return 0.0;
    if (s->period_s1 > 0.0 && s->n1 > 0) {
        double tp = t - s->start;
        if (tp >= 0 && tp <= s->period_s1 * s->n1) {
            double phase = tp - floor(tp / s->period_s1) * s->period_s1;
            if (phase >= 0 && phase <= s->duration) istim = -s->amplitude;
        }
    }
    if (istim == 0.0 && s->period_s2 > 0.0 && s->n2 > 0) {
        double t1 = s->start + s->period_s1 * s->n1;
        double tp = t - t1;
        if (tp >= 0 && tp <= s->period_s2 * s->n2) {
            double phase = tp - floor(tp / s->period_s2) * s->period_s2;
            if (phase >= 0 && phase <= s->duration) istim = -s->amplitude;
        }
    }
    return istim;
}

/* Foam::heaviside (src/ionicModels/BuenoOrovio/heaviside.H:39-48): int 1/0 */
static inline int oracle_heaviside(double x) { return x > 0 ? 1 : 0; }

/* tissueSelect (src/ionicModels/ToRORd_dynCl/ToRORd_dynCl_2023.H:558-568) */
static inline double oracle_tissue_select(int t, double endo, double mid, double epi)
{
    return (t == 3) ? endo : (t == 2) ? mid : epi;
}

void oracle_fatal(const char* what);

#ifdef __cplusplus
}
#endif
#endif
