// Compiles ONE of the reference's generated ionic-model headers verbatim
// (include path points into the reference tree; nothing is copied) and
// exports its functions under C names prefixed with REF_PREFIX.  Built by
// oracle/ref/build_ref.sh into oracle/_ref/ to pin the oracle's model code.
#include MODEL_HEADER

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)

extern "C" {
int CAT(REF_PREFIX, _sizes)(int* ns, int* na, int* nc)
{
    *ns = NUM_STATES; *na = NUM_ALGEBRAIC; *nc = NUM_CONSTANTS;
    return 0;
}
void CAT(REF_PREFIX, _init)(double* C, double* R, double* S, int tissue)
{
    Foam::dictionary d;
    CAT(MODEL_PREFIX, initConsts)(C, R, S, tissue, d);
}
static Foam::StimulusProtocol make_stim(const double* p)
{
    Foam::StimulusProtocol s;
    if (p) {
        s.stimStart = p[0]; s.stimPeriodS1 = p[1]; s.stimDuration = p[2];
        s.stimAmplitude = p[3]; s.nStim1 = (int)p[4]; s.stimPeriodS2 = p[5];
        s.nStim2 = (int)p[6];
    }
    return s;
}
void CAT(REF_PREFIX, _rates)(double t, double* C, double* R, double* S, double* A, int tissue,
                             int solve_vm, const double* stim)
{
    Foam::StimulusProtocol s = make_stim(stim);
    RATES_FN(t, C, R, S, A, tissue, solve_vm != 0, s);
}
void CAT(REF_PREFIX, _variables)(double t, double* C, double* R, double* S, double* A,
                                 int tissue, int solve_vm, const double* stim)
{
    Foam::StimulusProtocol s = make_stim(stim);
    VARS_FN(t, C, R, S, A, tissue, solve_vm != 0, s);
#ifdef VARS_FN2
    VARS_FN2(t, C, R, S, A, tissue, solve_vm != 0, s);
#endif
}
}
