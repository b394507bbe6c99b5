/*
 * GPUStepTask.hpp -- the NairnMPM-side binding of the GB300 explicit step.
 *
 * One MPMTask (NairnMPM/src/NairnMPM_Class/MPMTask.hpp) that takes the place
 * of the task chain NairnMPM::CreateTasks builds (NairnMPM.cpp:870-1110, from
 * InitializationTask to ResetElementsTask) and advances the analysis one step
 * per Execute() through the C ABI of include/nairn_mpm_gpu.h.  NairnMPM keeps
 * the XML input, the material objects, the particle generation, the time
 * step and the archives; the task packs their state into the ABI's plain
 * structs once, and writes the particle state back into mpm[] before every
 * step whose time the archiver will write.
 *
 * Compiled against the reference's own headers and objects by
 * oracle/ref/Makefile (target `gpu`), which links NairnMPM-gpu with
 * NairnMPMGPU (NairnMPMGPU.cpp) in place of the reference's main.
 */
#ifndef GPU_STEP_TASK_HPP
#define GPU_STEP_TASK_HPP

#include <vector>

#include "NairnMPM_Class/MPMTask.hpp"
#include "nairn_mpm_gpu.h"

class GPUStepTask : public MPMTask
{
    public:
        GPUStepTask(const char *name);
        virtual ~GPUStepTask();
        virtual bool Execute(int taskOption);

        // mpm[] <- device state (called by Execute before archive steps)
        void SyncToHost(void);

    private:
        void Check(int status, const char *where) const;
        void PackParticles(void);
        void UnpackParticles(void);

        MpmGpuCtx *ctx;
        int dim;
        std::vector<double> cols;       // the double columns of soa, one block
        std::vector<int32_t> matCol, elemCol;
        std::vector<int> historyCount;  // history doubles of each material
        std::vector<int> deviceMat;     // device material of each material (-1: a contact law)
        MpmGpuParticles soa;
        bool hostStale;                 // mpm[] behind the device
};

#endif
