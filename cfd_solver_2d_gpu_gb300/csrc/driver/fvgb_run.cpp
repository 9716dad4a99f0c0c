// fvgb_run: the headless driver loop over the C ABI, in place of
// U2NITS::CDriver::start (FVMR/src/drivers/CDriver.cpp:31-184) for the GPU step.
//
//   fvgb_run input.toml [--output DIR] [--device N] [--quiet]
//
// Reads input.toml (fvgb_params_read_toml, fvgb_run_config_read_toml); the mesh
// is <folder of input.toml>/<basic.filename>.su2.  With basic.continue it
// restarts from the newest pause_<filename>[n].dat in the output folder (the
// reference's rule, ContinueFileReader.cpp:24-53), else it starts from the
// initial field.  The loop follows CDriver::start and its signal packs
// (CDriver.cpp:202-263):
//   - print the residual at step 1 and every output.step_per_print steps;
//   - append a line (iteration, t, the four residuals, C_L and C_D of the
//     walls) to <filename>_hist.dat at step 1 and every
//     output.step_per_output_hist steps (FieldWriter::write_tecplot_hist_file,
//     FVMR/src/output/FieldWriter.cpp:211-262);
//   - write the Tecplot volume file <filename>[istep].dat and the boundary file
//     <filename>_tec_boundary.dat at step 1, every output.step_per_output_field
//     steps from output.start_output_field on, and at the stop
//     (FieldWriter.cpp:44-172, presets output.outputScheme_*_preset);
//   - stop at output.maxIteration, when the residual of rho falls to 1e-10
//     (U2NITS::Math::EPSILON), when the time reaches max_physical_time, or on
//     NaN; write pause_<filename>[istep].dat (istep as %04d) at the stop, or
//     nan_<filename>[istep].dat after a NaN.
// Between those events the device advances without host synchronisation
// (fvgb_step over the whole span).  Differences from the reference:
//   - The reference clamps dt so that t lands on T exactly and then keeps
//     stepping with dt = 0 until maxIteration. This driver stops at the first
//     output event at which t has reached T.
//   - Continue files carry 17 significant digits (the reference's 6).
//   - Node values in the Tecplot files come from the state after the step; the
//     reference's come from the primitive variables of the step's start.
// Exit status: 0 at a normal stop, 2 after NaN or an out-of-range state,
// 1 on any other error.
#include <sys/stat.h>

#include <algorithm>
#include <chrono>
#include <csignal>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "fvgb.h"

namespace {

// SIGINT / SIGTERM play the reference's ESC key (CDriver.cpp:244-249): the run stops at its
// next event and writes its pause file
volatile std::sig_atomic_t g_stop = 0;
void on_signal(int) { g_stop = 1; }

int report(const char* what) {
    std::fprintf(stderr, "fvgb_run: %s: %s\n", what, fvgb_last_error());
    return 1;
}

std::string folder_of(const std::string& path) {
    const size_t k = path.find_last_of('/');
    return k == std::string::npos ? std::string(".") : path.substr(0, k);
}

std::string step_tag(int istep) {
    char b[32];
    std::snprintf(b, sizeof b, "[%04d]", istep);  // COutput::updateFileName, FVMR/src/output/COutput.cpp:13-15
    return b;
}

int usage() {
    std::fprintf(stderr, "usage: fvgb_run input.toml [--output DIR] [--device N] [--quiet] [--snapshot-seconds S]\n");
    return 1;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2 || !std::strcmp(argv[1], "--help") || !std::strcmp(argv[1], "-h")) return usage();
    const std::string toml = argv[1];
    std::string out_dir = folder_of(toml) + "/output";
    int device = -1;
    bool quiet = false;
    // a pause file every so many seconds of wall time (CDriver.h:33-34, 30 minutes)
    double snapshot_seconds = 1800.0;
    for (int i = 2; i < argc; i++) {
        if (!std::strcmp(argv[i], "--output") && i + 1 < argc) out_dir = argv[++i];
        else if (!std::strcmp(argv[i], "--device") && i + 1 < argc) device = std::atoi(argv[++i]);
        else if (!std::strcmp(argv[i], "--quiet")) quiet = true;
        else if (!std::strcmp(argv[i], "--snapshot-seconds") && i + 1 < argc) snapshot_seconds = std::atof(argv[++i]);
        else return usage();
    }

    fvgb_params p;
    fvgb_run_config rc;
    char mesh_name[512];
    if (fvgb_params_read_toml(toml.c_str(), &p, mesh_name, sizeof mesh_name)) return report(toml.c_str());
    if (fvgb_run_config_read_toml(toml.c_str(), &rc)) return report(toml.c_str());
    if (device >= 0) p.device = device;
    if (std::strcmp(rc.mesh_file_type, "su2") != 0) {
        std::fprintf(stderr, "fvgb_run: basic.meshFileType = \"%s\": only su2 meshes are read\n", rc.mesh_file_type);
        return 1;
    }
    mkdir(out_dir.c_str(), 0755);
    const std::string name = rc.filename;

    // CInput::readField_1 (FVMR/src/input/CInput.cpp:102-120)
    fvgb_mesh* mesh = nullptr;
    std::vector<double> U;
    double t = 0.0;
    int istep = 0;
    bool restarted = false;
    if (rc.continue_run) {
        char path[4096];
        if (fvgb_find_continue_file(out_dir.c_str(), name.c_str(), path, sizeof path) == 0) {
            double cfl = -1.0;
            if (fvgb_read_continue(path, p.equation, &mesh, &t, &istep, &cfl)) return report(path);
            if (cfl >= 0.0) p.CFL = cfl;  // ContinueFileReader.cpp:98-100 keeps the saved CFL
            fvgb_mesh_soa soa;
            fvgb_mesh_view(mesh, &soa);
            U.resize(4 * (size_t)soa.num_element);
            if (fvgb_continue_state(mesh, U.data())) return report(path);
            restarted = true;
            if (!quiet) std::printf("continue from: %s (step %d, t = %.17g)\n", path, istep, t);
        } else if (!quiet) {
            std::printf("failed to read continue file (pause_*.dat), will read mesh file.\n");
        }
    }
    fvgb_mesh_soa soa;
    if (!restarted) {
        const std::string su2 = folder_of(toml) + "/" + name + ".su2";
        if (fvgb_mesh_read_su2(su2.c_str(), p.equation, p.mesh_scale, &mesh)) return report(su2.c_str());
        fvgb_mesh_view(mesh, &soa);
        U.resize(4 * (size_t)soa.num_element);
        if (fvgb_initial_field(&soa, &p, U.data())) return report("initial field");
    } else {
        fvgb_mesh_view(mesh, &soa);
    }

    fvgb_handle* h = nullptr;
    if (fvgb_create(&soa, &p, &h)) return report("fvgb_create");
    // time.strategy: the adaptive CFL of RoutineController, applied at each print event
    fvgb_cfl_controller* ctl_raw = nullptr;
    if (fvgb_cfl_controller_create(rc.time_strategy, &ctl_raw)) return report("time.strategy");
    std::unique_ptr<fvgb_cfl_controller, void (*)(fvgb_cfl_controller*)> ctl(ctl_raw, fvgb_cfl_controller_destroy);
    if (fvgb_set_state(h, U.data())) return report("fvgb_set_state");

    // write_tecplot_hist_file: the head when the file is new or the run did not restart
    const std::string hist_path = out_dir + "/" + name + "_hist.dat";
    bool hist_head = !restarted;
    if (FILE* probe = std::fopen(hist_path.c_str(), "r")) std::fclose(probe);
    else hist_head = true;
    FILE* hist = std::fopen(hist_path.c_str(), hist_head ? "w" : "a");
    if (!hist) {
        std::fprintf(stderr, "fvgb_run: cannot write %s\n", hist_path.c_str());
        return 1;
    }
    if (hist_head)
        std::fprintf(hist, "title= \"tecplot hist file\"\nvariables= \"Iteration\", \"physical_time\", \"R_1\", "
                           "\"R_2\", \"R_3\", \"R_4\", \"C_L\", \"C_D\"\nzone t= \"zone title\", f= point\n");
    std::vector<double> cd_set(soa.num_boundary > 0 ? soa.num_boundary : 1), cl_set(cd_set.size());
    auto write_fields = [&](int at) -> int {
        const std::string vol = out_dir + "/" + name + step_tag(at) + ".dat";
        const std::string bnd = out_dir + "/" + name + "_tec_boundary.dat";
        if (fvgb_write_tecplot_volume(h, vol.c_str(), "title", t, rc.volume_preset)) return report(vol.c_str());
        if (fvgb_write_tecplot_boundary(h, bnd.c_str(), t, rc.boundary_preset)) return report(bnd.c_str());
        return 0;
    };

    const double T = p.T_end;
    const int max_it = rc.max_iteration;
    const double kEpsilon = 1e-10;  // U2NITS::Math::EPSILON, FVMR/src/math/CommonValue.h
    int status = 0;
    const char* why = "maximum iteration reached";
    std::string final_prefix = "pause_";
    auto next_multiple = [](int after, int every) { return (after / every + 1) * every; };
    int last_field_step = -1;
    const auto t_start = std::chrono::steady_clock::now();
    std::signal(SIGINT, on_signal);
    std::signal(SIGTERM, on_signal);
    double last_snapshot = 0.0;
    while (istep < max_it) {
        // the next step at which CDriver::start would print or write (modifySignalPack1_output)
        int target = max_it;
        if (istep == 0) target = 1;
        target = std::min(target, next_multiple(istep, rc.step_per_print));
        target = std::min(target, next_multiple(istep, rc.step_per_output_hist));
        target = std::min(target, next_multiple(istep, rc.step_per_output_field));
        int rcs = fvgb_step(h, &t, T, target - istep);
        if (rcs == FVGB_ERR_NAN || rcs == FVGB_ERR_RANGE) {
            std::fprintf(stderr, "fvgb_run: %s near step %d\n", fvgb_last_error(), target);
            istep = target;
            status = 2;
            why = "NaN or out-of-range state detected";
            final_prefix = "nan_";
            break;
        }
        if (rcs) return report("fvgb_step");
        istep = target;
        double res[4];
        if (fvgb_residual(h, 0, res)) return report("fvgb_residual");
        const bool print = istep == 1 || istep % rc.step_per_print == 0;
        const bool write_hist = istep == 1 || istep % rc.step_per_output_hist == 0;
        const bool write_field =
            istep == 1 || (istep % rc.step_per_output_field == 0 && istep >= rc.start_output_field);
        if (print) {  // CDriver.cpp:115-125: the residual, then the CFL strategy, then the print
            int applied = 0;
            double cfl = p.CFL;
            if (fvgb_cfl_controller_apply(ctl.get(), res[0], istep, &cfl, &applied)) return report("time.strategy");
            if (applied && cfl != p.CFL) {
                p.CFL = cfl;
                if (fvgb_set_cfl(h, cfl)) return report("fvgb_set_cfl");
                if (!quiet) std::printf("step = %d\tresidual_rho = %.6e\tCFL = %.9g\n", istep, res[0], cfl);
            }
        }
        if (print && !quiet)
            std::printf("step = %d\tt = %.9g\tresidual_rho = %.6e\tresidual_rhou = %.6e\tresidual_rhov = %.6e\t"
                        "residual_rhoE = %.6e\n",
                        istep, t, res[0], res[1], res[2], res[3]);
        if (write_hist) {
            double cdw = 0.0, clw = 0.0;
            if (fvgb_boundary_forces(h, cd_set.data(), cl_set.data(), &cdw, &clw)) return report("forces");
            std::fprintf(hist, "%d %e %e %e %e %e %e %e\n", istep, t, res[0], res[1], res[2], res[3], clw, cdw);
            std::fflush(hist);
        }
        if (write_field) {
            if (write_fields(istep)) return 1;
            last_field_step = istep;
        }
        // modifySignalPack1_output's snapshot (CDriver.cpp:227-232): a pause file once the wall
        // time since the last one exceeds the cool-down, checked here at each event
        const double now = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
        if (now - last_snapshot > snapshot_seconds) {
            last_snapshot = now;
            if (fvgb_get_state(h, U.data())) return report("fvgb_get_state");
            const std::string snap = out_dir + "/pause_" + name + step_tag(istep) + ".dat";
            if (fvgb_write_continue(mesh, snap.c_str(), t, istep, p.CFL, U.data())) return report(snap.c_str());
        }
        // modifySignalPack2_pause (CDriver.cpp:230-263)
        if (std::isnan(res[0])) {
            status = 2;
            why = "NaN detected";
            final_prefix = "nan_";
            break;
        }
        if (g_stop) {
            why = "stopped by a signal";
            break;
        }
        if (t >= T) {
            why = "physical time reached";
            break;
        }
        if (res[0] <= kEpsilon) {
            why = "steady state reached";
            break;
        }
    }
    std::fclose(hist);
    // every stop writes the field too (modifySignalPack2_pause sets b_writeTecplot)
    if (last_field_step != istep && write_fields(istep)) return 1;

    if (fvgb_get_state(h, U.data())) return report("fvgb_get_state");
    const std::string cont = out_dir + "/" + final_prefix + name + step_tag(istep) + ".dat";
    if (fvgb_write_continue(mesh, cont.c_str(), t, istep, p.CFL, U.data())) return report(cont.c_str());
    if (!quiet) std::printf("%s at step %d, t = %.17g; wrote %s\n", why, istep, t, cont.c_str());
    fvgb_destroy(h);
    fvgb_mesh_free(mesh);
    return status;
}
