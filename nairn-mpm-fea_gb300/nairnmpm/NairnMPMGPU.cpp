/*
 * NairnMPMGPU.cpp -- NairnMPM with the explicit step on the GB300.
 *
 * NairnMPMGPU is the reference's NairnMPM analysis (NairnMPM/src/
 * NairnMPM_Class/NairnMPM.cpp) with one change: after CMPreparations has
 * read the input, generated the particles, found the time step and built the
 * task chain, the chain is replaced by one GPUStepTask.  main() here does
 * what the reference's main (Common/System/main.cpp) does for an MPM run --
 * create the analysis, read the XML file, run it -- with this class; the
 * command line is the reference's (-np N is accepted and passed on, other
 * options refused).
 */
#include "stdafx.h"

#include <cstdio>
#include <cstring>

#include "NairnMPM_Class/NairnMPM.hpp"
#include "Exceptions/CommonException.hpp"
#include "nairnmpm/GPUStepTask.hpp"

extern MPMTask *firstMPMTask;

class NairnMPMGPU : public NairnMPM
{
    public:
        virtual void CMPreparations(void)
        {	NairnMPM::CMPreparations();
            firstMPMTask = (MPMTask *)new GPUStepTask("GB300 explicit step (mpmgpu_step)");
        }
};

int main(int argc, const char *argv[])
{
    fmobj = new NairnMPMGPU();
    int numProcs = 1, arg = 1;
    for(; arg < argc && argv[arg][0] == '-'; arg++)
    {	if(strcmp(argv[arg], "-np") == 0 && arg + 1 < argc)
            sscanf(argv[++arg], "%d", &numProcs);
        else
        {	fprintf(stderr, "usage: %s [-np N] input.xml\n", argv[0]);
            return NoInputErr;
        }
    }
    if(arg + 1 != argc)
    {	fprintf(stderr, "usage: %s [-np N] input.xml\n", argv[0]);
        return NoInputErr;
    }
    fmobj->SetNumberOfProcessors(numProcs);
    int status = fmobj->ReadFile(argv[arg], false);
    if(status != noErr) return status;
    try
    {	fmobj->StartAnalysis(false);
    }
    catch(CommonException &err)
    {	err.Display(fmobj->mstep, mtime);
        return err.ErrorCode();
    }
    catch(CommonException *err)
    {	err->Display(fmobj->mstep, mtime);
        return err->ErrorCode();
    }
    catch(const char *msg)
    {	fprintf(stderr, "%s\n", msg);
        return AnalysisErr;
    }
    return noErr;
}
