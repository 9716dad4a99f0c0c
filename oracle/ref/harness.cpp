// Headless driver for the reference's own CPU step path (test infrastructure:
// only the parity tests and the fixture generator under tests/golden run it).
//
// It replaces the parts of U2NITS::CDriver::start (FVMR/src/drivers/CDriver.cpp:
// 44-80) that lead up to the step loop: read input.toml through the
// reference's TomlFileManager, read and assemble the .su2 mesh through
// SU2MeshReader/FVM_2D, set the initial field with FieldInitializer, build
// the SoA arrays through GPUSolver2/OldDataConverter, and then step with the
// reference's own functions:
//   euler      CIteration::iteration_host with time_advance 3101
//              (FVMR/src/time/CIteration.cpp:28-80)
//   rk3lit     CIteration::iteration_host with time_advance 3103, the
//              reference's RK3 exactly as written (Evolve.cpp:25-96)
//   rk3        classical (Kutta) RK3 with the weights of Evolve.cpp:26-37,
//              each stage evaluated by the reference's calculateFunctionF on
//              the solver singleton (Evolve.cpp:98-112), the double-Mach-
//              reflection clock set as CIteration.cpp:60-62 and Evolve.cpp:43-77
//              set it (t; then dt 0, dt, 0.5 dt for the three stages)
//   ssprk3     Shu-Osher SSP-RK3 built the same way (new code 3104)
//   rhs        one calculateFunctionF on the initial field, plus its dt
//   mesh       assembly and initial field only
//   output     nsteps forward-Euler steps, then the reference's own field output of
//              the final state: FieldWriter::update_nodeField (node values dumped),
//              write_tecplot_volume_file / write_tecplot_boundary_file and one
//              write_tecplot_hist_file line (residuals 1, 2, 3, 4), written to
//              <out>.volume.dat, <out>.boundary.dat and <out>.hist.dat
//              (FVMR/src/output/FieldWriter.cpp:44-262, 364-453)
//   continue   the newest pause_<basic.filename>[n].dat of the folder given in
//              place of the mesh, read by ContinueFileReader::readContinueFile_1
//              (FVMR/src/input/ContinueFileReader.cpp:19-158): mesh and field only
// and writes every SoA array, the final field, the per-step dt and the residual
// norms of the last residual (get_residual_host, all three norms) to a small
// binary file ("FVMRDUMP" + named arrays) that tests read with numpy.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "global/GlobalPara.h"
#include "input/TomlFileManager.h"
#include "input/SU2MeshReader.h"
#include "input/FieldInitializer.h"
#include "input/ContinueFileReader.h"
#include "output/FieldWriter.h"
#include "solvers/GPUSolver2.h"
#include "time/CIteration.h"
#include "time/CalculateDt.h"
#include "time/Evolve.h"
#include "space/restrict/Restrict.h"
#include "output/residual/Residual.h"
#include "boundary_condition/CBoundaryDoubleShockReflect.h"

namespace {

struct Dump {
    FILE* f = nullptr;
    explicit Dump(const char* path) {
        f = std::fopen(path, "wb");
        if (!f) { std::perror(path); std::exit(2); }
        std::fwrite("FVMRDUMP", 1, 8, f);
    }
    ~Dump() { if (f) std::fclose(f); }
    void put(const char* name, char code, const void* data, long long count, int elsize) {
        char nm[32] = {0};
        std::strncpy(nm, name, 31);
        std::fwrite(nm, 1, 32, f);
        std::fwrite(&code, 1, 1, f);
        std::fwrite(&count, sizeof(count), 1, f);
        if (count) std::fwrite(data, elsize, (size_t)count, f);
    }
    void i32(const char* name, const int* p, long long n) { put(name, 'i', p, n, 4); }
    void f64(const char* name, const std::vector<double>& v) { put(name, 'd', v.data(), (long long)v.size(), 8); }
    template <class T>
    void rows(const char* name, T* const* rowsp, int nrow, int n) {
        std::vector<double> v((size_t)nrow * n);
        for (int r = 0; r < nrow; r++)
            for (int i = 0; i < n; i++) v[(size_t)r * n + i] = (double)rowsp[r][i];
        f64(name, v);
    }
    void irows(const char* name, int* const* rowsp, int nrow, int n) {
        std::vector<int> v((size_t)nrow * n);
        for (int r = 0; r < nrow; r++)
            for (int i = 0; i < n; i++) v[(size_t)r * n + i] = rowsp[r][i];
        i32(name, v.data(), (long long)v.size());
    }
};

void copy_field(myfloat* const* src, std::vector<double>& dst, int n) {
    dst.resize((size_t)4 * n);
    for (int j = 0; j < 4; j++)
        for (int i = 0; i < n; i++) dst[(size_t)j * n + i] = (double)src[j][i];
}

void load_field(const std::vector<double>& src, myfloat* const* dst, int n) {
    for (int j = 0; j < 4; j++)
        for (int i = 0; i < n; i++) dst[j][i] = (myfloat)src[(size_t)j * n + i];
}

// One evaluation of the reference residual on the solver singleton: the
// state is placed in the singleton's U because calculateFluxHost reads the
// singleton (FVMR/src/space/Flux.cpp:394-412).
void residual(GPU::GPUSolver2& s, const std::vector<double>& U, std::vector<double>& R) {
    const int n = s.element_host.num_element;
    load_field(U, s.elementField_host.U, n);
    U2NITS::Time::calculateFunctionF(s.element_host, s.node_host, s.edge_host, s.elementField_host);
    copy_field(s.elementField_host.Flux, R, n);
}

// The reference's own residual norms of the singleton's last residual (elementField_host.Flux),
// U2NITS::Output::get_residual_host (FVMR/src/output/residual/Residual.cpp:4-43), as
// GPUSolver2::updateResidualVector (GPUSolver2.cpp:294-296) asks for them: rows L-infinity,
// L1, L2 (the NormType order), columns the four conserved variables.
std::vector<double> residual_norms(GPU::GPUSolver2& s) {
    std::vector<double> out;
    const U2NITS::Output::NormType kinds[3] = {U2NITS::Output::normType_infinity, U2NITS::Output::normType_1,
                                               U2NITS::Output::normType_2};
    for (U2NITS::Output::NormType k : kinds) {
        myfloat r[4] = {0, 0, 0, 0};
        U2NITS::Output::get_residual_host(s.elementField_host, r, k);
        for (int v = 0; v < 4; v++) out.push_back((double)r[v]);
    }
    return out;
}

myfloat global_dt(GPU::GPUSolver2& s) {
    CIteration::update_host_ruvp_Uold(s.elementField_host.U, s.elementField_host.ruvp, s.elementField_host.Uold,
                                      s.elementField_host.num, GlobalPara::constant::gamma);
    return U2NITS::Time::get_global_dt_host(GlobalPara::constant::gamma, GlobalPara::constant::Pr, GlobalPara::time::CFL,
                                            GlobalPara::constant::R, s.elementFieldVariable_dt_host, s.element_host,
                                            s.edge_host, s.elementField_host, GlobalPara::physicsModel::equation);
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 6) {
        std::fprintf(stderr, "usage: %s input.toml mesh.su2 mode nsteps out.bin\n", argv[0]);
        return 2;
    }
    const std::string toml = argv[1], mesh = argv[2], mode = argv[3];
    const int nsteps = std::atoi(argv[4]);
    const char* out = argv[5];

    TomlFileManager::getInstance()->readTomlFile(toml);
    GlobalPara::basic::useGPU = 0;
    if (mode == "continue") {
        // CInput::readField_1 with basic.continue: the newest pause_<basic.filename>[n].dat in
        // the folder given in place of the mesh; the field initialiser is not called then
        setenv("FVMR_REF_OUTDIR", mesh.c_str(), 1);
        if (ContinueFileReader::readContinueFile_1() != 0) {
            std::fprintf(stderr, "no continue file in %s\n", mesh.c_str());
            return 5;
        }
    } else {
        SU2MeshReader::read_mesh_and_process(mesh, true);
        FieldInitializer::getInstance()->setInitialAndBoundaryCondition();
    }

    GPU::GPUSolver2 s;
    s.allocateMemory();
    s.initializeData();
    const int N = s.element_host.num_element, E = s.edge_host.num_edge, V = s.node_host.num_node;
    const int NB = s.boundary_host.size;

    Dump d(out);
    int sizes[4] = {N, E, V, NB};
    d.i32("sizes", sizes, 4);
    d.rows("node_xy", s.node_host.xy, 2, V);
    d.irows("elem_nodes", s.element_host.nodes, 4, N);
    d.irows("elem_edges", s.element_host.edges, 4, N);
    d.irows("elem_nbrs", s.element_host.neighbors, 4, N);
    d.rows("elem_xy", s.element_host.xy, 2, N);
    d.rows("elem_vol", &s.element_host.volume, 1, N);
    d.irows("edge_nodes", s.edge_host.nodes, 2, E);
    d.i32("edge_L", s.edge_host.elementL, E);
    d.i32("edge_R", s.edge_host.elementR, E);
    d.i32("edge_set", s.edge_host.setID, E);
    d.i32("edge_pair", s.edge_host.periodicPair, E);
    d.rows("edge_len", &s.edge_host.length, 1, E);
    d.rows("edge_dist", &s.edge_host.distanceOfElements, 1, E);
    d.rows("edge_xy", s.edge_host.xy, 2, E);
    d.rows("edge_normal", s.edge_host.normal, 2, E);
    d.i32("bc_type", s.boundary_host.type, NB);
    d.rows("U0", s.elementField_host.U, 4, N);
    std::vector<double> params = {
        (double)GlobalPara::constant::gamma, (double)GlobalPara::constant::R, (double)GlobalPara::constant::Pr,
        (double)GlobalPara::constant::mu0, (double)GlobalPara::constant::T0, (double)GlobalPara::constant::Re,
        (double)GlobalPara::time::CFL, (double)GlobalPara::time::max_physical_time,
        (double)GlobalPara::boundaryCondition::_2D::inf::ruvp[0], (double)GlobalPara::boundaryCondition::_2D::inf::ruvp[1],
        (double)GlobalPara::boundaryCondition::_2D::inf::ruvp[2], (double)GlobalPara::boundaryCondition::_2D::inf::ruvp[3],
        (double)GlobalPara::boundaryCondition::_2D::inlet::ruvp[0], (double)GlobalPara::boundaryCondition::_2D::inlet::ruvp[1],
        (double)GlobalPara::boundaryCondition::_2D::inlet::ruvp[2], (double)GlobalPara::boundaryCondition::_2D::inlet::ruvp[3],
        (double)GlobalPara::boundaryCondition::_2D::outlet::ruvp[0], (double)GlobalPara::boundaryCondition::_2D::outlet::ruvp[1],
        (double)GlobalPara::boundaryCondition::_2D::outlet::ruvp[2], (double)GlobalPara::boundaryCondition::_2D::outlet::ruvp[3]};
    d.f64("params", params);
    std::vector<double> cont = {(double)GlobalPara::time::t_previous, (double)GlobalPara::time::istep_previous,
                                (double)GlobalPara::time::CFL};
    d.f64("continue", cont);
    if (mode == "mesh" || mode == "continue") return 0;

    std::vector<double> U0, R;
    copy_field(s.elementField_host.U, U0, N);

    if (mode == "rhs") {
        std::vector<double> dt = {(double)global_dt(s)};
        std::vector<double> alpha(s.elementFieldVariable_dt_host.alphaC, s.elementFieldVariable_dt_host.alphaC + N);
        residual(s, U0, R);
        d.f64("rhs", R);
        d.f64("residual_norms", residual_norms(s));
        d.rows("grad_x", s.elementField_host.Ux, 4, N);
        d.rows("grad_y", s.elementField_host.Uy, 4, N);
        d.f64("dt", dt);
        d.f64("alphaC", alpha);
        return 0;
    }

    myfloat t = 0;
    const myfloat T = GlobalPara::time::max_physical_time;
    std::vector<double> dts;
    std::vector<double> k1, k2, k3, Us;
    for (int step = 0; step < nsteps; step++) {
        if (mode == "euler" || mode == "rk3lit" || mode == "output") {
            GlobalPara::time::time_advance = (mode == "rk3lit") ? _EVO_rk3 : _EVO_explicit;
            myfloat t0 = t;
            CIteration::iteration_host(t, T, &s);
            dts.push_back((double)(t - t0));
            continue;
        }
        myfloat dt = global_dt(s);
        if (t + dt > T) dt = T - t;
        CBoundaryDoubleShockReflect* dsr = CBoundaryDoubleShockReflect::getInstance();
        dsr->set_t(t);
        dsr->set_dt(0.0);
        t += dt;
        dts.push_back((double)dt);
        copy_field(s.elementField_host.U, U0, N);
        const size_t M = (size_t)4 * N;
        Us.resize(M);
        if (mode == "rk3") {
            // weights and stage points of FVMR/src/time/Evolve.cpp:58-86
            residual(s, U0, k1);
            for (size_t i = 0; i < M; i++) Us[i] = (double)((myfloat)U0[i] + 0.5 * dt * (myfloat)k1[i]);
            dsr->set_dt(dt);
            residual(s, Us, k2);
            for (size_t i = 0; i < M; i++)
                Us[i] = (double)((myfloat)U0[i] - dt * (myfloat)k1[i] + 2.0 * dt * (myfloat)k2[i]);
            dsr->set_dt(0.5 * dt);
            residual(s, Us, k3);
            const myfloat dt_on_6 = dt / 6.0;
            for (size_t i = 0; i < M; i++)
                Us[i] = (double)((myfloat)U0[i] + dt_on_6 * ((myfloat)k1[i] + 4 * (myfloat)k2[i] + (myfloat)k3[i]));
        } else if (mode == "ssprk3") {
            // Shu-Osher form: U1 = U0 + dt L(U0); U2 = 3/4 U0 + 1/4 (U1 + dt L(U1));
            // U3 = 1/3 U0 + 2/3 (U2 + dt L(U2))
            residual(s, U0, k1);
            std::vector<double> U1(M), U2(M);
            for (size_t i = 0; i < M; i++) U1[i] = (double)((myfloat)U0[i] + dt * (myfloat)k1[i]);
            dsr->set_dt(dt);
            residual(s, U1, k2);
            for (size_t i = 0; i < M; i++)
                U2[i] = (double)(0.75 * (myfloat)U0[i] + 0.25 * ((myfloat)U1[i] + dt * (myfloat)k2[i]));
            dsr->set_dt(0.5 * dt);
            residual(s, U2, k3);
            for (size_t i = 0; i < M; i++)
                Us[i] = (double)((1.0 / 3.0) * (myfloat)U0[i] + (2.0 / 3.0) * ((myfloat)U2[i] + dt * (myfloat)k3[i]));
        } else {
            std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
            return 2;
        }
        load_field(Us, s.elementField_host.U, N);
        U2NITS::Space::Restrict::modifyElementFieldU2d(s.element_host, s.elementField_host);
    }
    d.rows("U", s.elementField_host.U, 4, N);
    d.f64("residual_norms", residual_norms(s));
    if (mode == "output") {
        // the writers read ruvp: refresh it from the final state
        CIteration::update_host_ruvp_Uold(s.elementField_host.U, s.elementField_host.ruvp, s.elementField_host.Uold, N,
                                          GlobalPara::constant::gamma);
        // the output schemes were read with input.toml and the node arrays allocated by
        // GPUSolver2::allocateMemory (GPUSolver2.cpp:97)
        FieldWriter* w = FieldWriter::getInstance();
        w->update_nodeField();
        d.rows("node_ruvp", s.outputNodeField.ruvp, 4, V);
        d.f64("node_Cp", std::vector<double>(s.outputNodeField.Cp.begin(), s.outputNodeField.Cp.end()));
        d.f64("node_Ma", std::vector<double>(s.outputNodeField.Ma.begin(), s.outputNodeField.Ma.end()));
        const std::string base = out;
        w->write_tecplot_volume_file(t, base + ".volume.dat", "title", s.node_host, s.element_host, s.outputNodeField);
        w->write_tecplot_boundary_file(t, base + ".boundary.dat", s.node_host, s.edge_host, s.outputNodeField,
                                       s.boundary_host_new);
        myfloat res[4] = {1, 2, 3, 4};
        w->write_tecplot_hist_file(base + ".hist.dat", nsteps, t, res, s.edge_host, s.outputNodeField,
                                   s.boundary_host_new);
    }
    d.f64("dts", dts);
    std::vector<double> tt = {(double)t};
    d.f64("t", tt);
    return 0;
}
