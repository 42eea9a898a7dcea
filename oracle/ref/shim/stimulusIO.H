// Stand-in for src/genericWriter/stimulusIO.H: the StimulusProtocol fields
// (stimulusIO.H:32-53) and stimulusIO::computeStimulus restated from
// stimulusIO.C:238-286, so that the generated model headers link.
#pragma once
#include "scalar.H"
#include "dictionary.H"
namespace Foam {
struct StimulusProtocol {
    scalar stimStart = 0, stimPeriodS1 = 0, stimDuration = 0, stimAmplitude = 0;
    label nStim1 = 0;
    scalar stimPeriodS2 = 0;
    label nStim2 = 0;
};
struct stimulusIO {
    static scalar computeStimulus(scalar t, const StimulusProtocol& s) {
        scalar I = 0.0;
        if (s.stimPeriodS1 > 0.0 && s.nStim1 > 0) {
            scalar tp = t - s.stimStart;
            if (tp >= 0 && tp <= s.stimPeriodS1 * s.nStim1) {
                scalar ph = tp - std::floor(tp / s.stimPeriodS1) * s.stimPeriodS1;
                if (ph >= 0 && ph <= s.stimDuration) I = -s.stimAmplitude;
            }
        }
        if (I == 0.0 && s.stimPeriodS2 > 0.0 && s.nStim2 > 0) {
            scalar t1 = s.stimStart + s.stimPeriodS1 * s.nStim1;
            scalar tp = t - t1;
            if (tp >= 0 && tp <= s.stimPeriodS2 * s.nStim2) {
                scalar ph = tp - std::floor(tp / s.stimPeriodS2) * s.stimPeriodS2;
                if (ph >= 0 && ph <= s.stimDuration) I = -s.stimAmplitude;
            }
        }
        return I;
    }
};
}
