// Drives include/dgx_dgfem.hpp the way dgfem's own code would: a shared DGMesh built from
// vertex/element arrays and boundary edges, periodic pairing, a DG space, a solver built from
// (mesh, gamma), and states held as std::vector of Np x 4 matrices (the layer's own dense type
// here; dgfem's Eigen::MatrixXd when Eigen is on the include path).  Reads its inputs from files written by
// tests/test_gpu_cpp_layer.py and writes the results next to them as raw doubles.
//   usage: test_dgfem_compat <dir>
#include <dgx_dgfem.hpp>

#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

using Mat = dgx_dgfem::MatrixXd;

template <class T>
static std::vector<T> read_all(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    f.seekg(0, std::ios::end);
    const size_t n = (size_t)f.tellg() / sizeof(T);
    f.seekg(0);
    std::vector<T> v(n);
    f.read(reinterpret_cast<char*>(v.data()), n * sizeof(T));
    return v;
}

static void write_state(const std::string& path, const std::vector<Mat>& u) {
    std::ofstream f(path, std::ios::binary);
    for (const Mat& m : u)
        for (long i = 0; i < m.rows(); ++i)
            for (long v = 0; v < m.cols(); ++v) {
                const double x = m(i, v);
                f.write(reinterpret_cast<const char*>(&x), sizeof(x));
            }
}

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    const std::string dir = argv[1];
    const std::vector<double> V = read_all<double>(dir + "/vertices.bin");
    const std::vector<int> E = read_all<int>(dir + "/elements.bin");
    const std::vector<int> B = read_all<int>(dir + "/bedges.bin");
    const std::vector<double> U = read_all<double>(dir + "/state.bin");
    const std::vector<double> P = read_all<double>(dir + "/params.bin");  // order, dt, nvpe, basis
    const int order = (int)P[0];
    const double dt = P[1];
    const int nvpe = (int)P[2], basis = (int)P[3];

    Mat verts((int)V.size() / 2, 2);
    for (long i = 0; i < verts.rows(); ++i) { verts(i, 0) = V[2 * i]; verts(i, 1) = V[2 * i + 1]; }
    dgx_dgfem::MatrixXi elems((int)E.size() / nvpe, nvpe);
    for (long i = 0; i < elems.rows(); ++i)
        for (int k = 0; k < nvpe; ++k) elems(i, k) = E[(size_t)nvpe * i + k];
    std::map<int, std::vector<std::pair<int, int>>> edges;
    for (size_t k = 0; k + 2 < B.size(); k += 3) edges[B[k]].push_back({B[k + 1], B[k + 2]});
    const std::map<std::string, int> tags = {{"Bottom", 2}, {"Right", 3}, {"Top", 4}, {"Left", 5}};

    try {
        auto mesh = std::make_shared<dgx_dgfem::DGMesh>(verts, elems, dgx_dgfem::VectorXi(elems.rows()), tags, edges);
        const std::string type = nvpe == 4 ? "quad" : "triangle";
        if (mesh->get_element_type() != type) return 4;
        mesh->set_periodic_boundaries("Left", "Right");
        mesh->set_periodic_boundaries("Bottom", "Top");
        mesh->initialize_dg_space(std::make_shared<dgx_dgfem::DGSpace>(type, order, basis), 4);
        dgx_dgfem::EulerDGSolver solver(mesh, 1.4);
        // the assembler on its own, as DGAssembler(mesh, weak_form)
        dgx_dgfem::DGAssembler assembler(mesh, std::make_shared<dgx_dgfem::EulerWeakFormulation>(1.4));
        const int ne = solver.n_elements(), np = solver.n_basis();
        std::vector<Mat> u(ne, Mat(np, 4));
        for (int e = 0; e < ne; ++e)
            for (int i = 0; i < np; ++i)
                for (int v = 0; v < 4; ++v) u[e](i, v) = U[((size_t)e * np + i) * 4 + v];

        std::vector<Mat> R, R2;
        solver.assemble_euler_residual(u, R);
        assembler.assemble_euler_residual(u, R2);
        write_state(dir + "/residual.bin", R);
        write_state(dir + "/residual_assembler.bin", R2);
        write_state(dir + "/minv.bin", solver.apply_mass_inv(R));
        write_state(dir + "/rk3.bin", solver.time_step_ssp_rk3(u, dt));
        const double cfl = solver.compute_max_cfl(u, dt);
        const auto rr = solver.compute_density_range(u);
        std::ofstream(dir + "/monitors.txt") << std::hexfloat << cfl << " " << rr.first << " " << rr.second << "\n";

        bool threw = false;  // dgfem-style exception on a malformed state
        try {
            std::vector<Mat> bad(ne - 1, Mat(np, 4));
            solver.assemble_euler_residual(bad, R);
        } catch (const std::invalid_argument&) {
            threw = true;
        }
        if (!threw) return 3;
    } catch (const std::exception& ex) {
        std::cerr << "error: " << ex.what() << "\n";
        return 1;
    }
    return 0;
}
