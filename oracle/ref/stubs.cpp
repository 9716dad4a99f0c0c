// Link-time stand-ins for the reference symbols that the CPU step path names
// but never needs: logging, console/driver singletons, output writers and the
// GPU launchers (this build runs `CIteration::iteration_host` only).
// Nothing here computes anything on the hot path; every GPU launcher aborts
// loudly if it is ever reached.  Oracle build only (test infrastructure).
#include <cstdio>
#include <cstdlib>
#include <string>
#include <new>

#include <dirent.h>

#include <algorithm>
#include <vector>

#include "output/LogWriter.h"
#include "global/FilePathManager.h"
#include "global/CExit.h"
#include "output/FieldWriter.h"
#include "drivers/RoutineController.h"
#include "drivers/CDriver.h"
#include "gpu/datatype/Datatype.h"
#include "time/CalculateDtGPU.h"
#include "time/EvolveGPU.h"
#include "space/restrict/RestrictGPU.h"
#include "math/PhysicalKernelGPU.h"
#include "math/BasicAlgorithmGPU.h"

static bool quiet() { return std::getenv("FVMR_REF_VERBOSE") == nullptr; }

// The harness's continue mode: ContinueFileReader looks for pause files in the
// output folder, which here is the folder named by FVMR_REF_OUTDIR.
FilePathManager* FilePathManager::getInstance() {
    static FilePathManager* p = new FilePathManager();
    return p;
}
void FilePathManager::initialzeVariables() {
    const char* d = std::getenv("FVMR_REF_OUTDIR");
    m_outputDirectory = std::string(d ? d : ".") + "/";
}
std::vector<std::string> FilePathManager::getFiles(std::string path) {
    std::vector<std::string> out;
    if (DIR* d = opendir(path.c_str())) {
        while (dirent* e = readdir(d))
            if (e->d_name[0] != '.') out.push_back(e->d_name);
        closedir(d);
    }
    std::sort(out.begin(), out.end());
    return out;
}

void LogWriter::log(std::string, LogLevel) {}
void LogWriter::print(std::string c, LogLevel) { if (!quiet()) std::fputs(c.c_str(), stderr); }
void LogWriter::logAndPrint(std::string c, LogLevel, LogLevel) { if (!quiet()) std::fputs(c.c_str(), stderr); }
void LogWriter::logDebug(std::string) {}
void LogWriter::printDebug(std::string) {}
void LogWriter::logAndPrintDebug(std::string) {}
void LogWriter::logError(std::string c) { std::fprintf(stderr, "[ref error] %s", c.c_str()); }
void LogWriter::printError(std::string c) { std::fprintf(stderr, "[ref error] %s", c.c_str()); }
void LogWriter::logAndPrintError(std::string c) { std::fprintf(stderr, "[ref error] %s", c.c_str()); }
void LogWriter::logWarning(std::string) {}
void LogWriter::logAndPrintWarning(std::string) {}

void CExit::saveAndExit(int code) {
    std::fprintf(stderr, "[ref] saveAndExit(%d)\n", code);
    std::exit(code == 0 ? 3 : code);
}
void CExit::pressAnyKeyToExit() {
    std::fprintf(stderr, "[ref] pressAnyKeyToExit\n");
    std::exit(4);
}

// Singletons whose members the configuration reader writes (show_gui, ...):
// zeroed storage of the right size and alignment stands in for the object.
alignas(64) static unsigned char g_driver_storage[sizeof(U2NITS::CDriver)];
U2NITS::CDriver* U2NITS::CDriver::getInstance() {
    return reinterpret_cast<U2NITS::CDriver*>(g_driver_storage);
}
alignas(64) static unsigned char g_routine_storage[sizeof(RoutineController)];
RoutineController* RoutineController::getInstance() {
    return reinterpret_cast<RoutineController*>(g_routine_storage);
}
void RoutineController::setStrategy(int) {}

[[noreturn]] static void no_gpu(const char* what) {
    std::fprintf(stderr, "[ref] GPU function %s reached in the CPU oracle build\n", what);
    std::abort();
}
myint GPU::ReduceHelper::get_dev_output_length(myint) { no_gpu("ReduceHelper"); }
myint GPU::ReduceHelper::get_next_power_2_number(myint) { no_gpu("ReduceHelper"); }
void GPU::NodeSoA::cuda_memcpy(NodeSoA*, const NodeSoA*, cudaMemcpyKind) { no_gpu("NodeSoA::cuda_memcpy"); }
void GPU::ElementSoA::cuda_memcpy(ElementSoA*, const ElementSoA*, cudaMemcpyKind) { no_gpu("ElementSoA::cuda_memcpy"); }
void GPU::ElementFieldSoA::cuda_memcpy(ElementFieldSoA*, const ElementFieldSoA*, cudaMemcpyKind) { no_gpu("ElementFieldSoA::cuda_memcpy"); }
void GPU::EdgeSoA::cuda_memcpy(EdgeSoA*, const EdgeSoA*, cudaMemcpyKind) { no_gpu("EdgeSoA::cuda_memcpy"); }
void GPU::BoundarySetMap::cuda_memcpy(BoundarySetMap*, const BoundarySetMap*, cudaMemcpyKind) { no_gpu("BoundarySetMap::cuda_memcpy"); }
void GPU::Math::assign_elements_in_array_device(myint, myint, myfloat*, myfloat) { no_gpu("assign_elements_in_array_device"); }
void GPU::Math::update_ruvp_Uold_device_2(GPU::ElementFieldSoA&, myfloat) { no_gpu("update_ruvp_Uold_device_2"); }
void GPU::Space::Restrict::modifyElementFieldU2d_device(GPU::ElementSoA&, GPU::ElementFieldSoA&, myfloat) { no_gpu("modifyElementFieldU2d_device"); }
void GPU::Time::evolve_explicit_globaltimestep_device(myfloat, GPU::ElementSoA&, GPU::NodeSoA&, GPU::EdgeSoA&, GPU::ElementFieldSoA&) { no_gpu("evolve_explicit_globaltimestep_device"); }
void GPU::Time::evolve_explicit_localtimestep_device(GPU::ElementSoA&, GPU::NodeSoA&, GPU::EdgeSoA&, GPU::ElementFieldSoA&, GPU::ElementFieldVariable_dt&) { no_gpu("evolve_explicit_localtimestep_device"); }
void GPU::Time::get_global_dt_device(myfloat, myfloat, myfloat, myfloat, myfloat, GPU::ElementFieldVariable_dt&, GPU::ElementSoA&, GPU::EdgeSoA&, GPU::ElementFieldSoA&, int) { no_gpu("get_global_dt_device"); }
void GPU::Time::get_local_dt_device(myfloat, myfloat, myfloat, myfloat, myfloat, GPU::ElementFieldVariable_dt&, GPU::ElementSoA&, GPU::EdgeSoA&, GPU::ElementFieldSoA&, int) { no_gpu("get_local_dt_device"); }
void __getLastCudaError(const char* msg, const char*, const int) { no_gpu(msg); }
