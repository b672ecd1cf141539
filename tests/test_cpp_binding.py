"""The C++ host binding (include/xpbd_gpu_solver.hpp) compiles against mock
reference types (no Eigen), links to libxpbd_gpu.so and runs: without a GPU it
must surface XPBD_ERR_NO_DEVICE as an exception; with one it solves."""
import os
import subprocess
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = textwrap.dedent(r"""
    #include <cstdio>
    #include <vector>
    #include "xpbd_gpu_solver.hpp"

    // minimal stand-ins for Geometry::Mesh / TetMesh / XPBDMeshObject_
    struct Mat { std::vector<double> v; double* data() { return v.data(); } const double* data() const { return v.data(); } };
    struct IMat { std::vector<int> v; const int* data() const { return v.data(); } };
    struct Mesh {
        Mat X; IMat F;
        int numVertices() const { return (int)X.v.size() / 3; }
        int numFaces() const { return (int)F.v.size() / 3; }
        Mat& vertices() { return X; }
        const IMat& faces() const { return F; }
    };
    struct TetMesh { IMat E; int numElements() const { return (int)E.v.size() / 4; } const IMat& elements() const { return E; } };
    struct Obj {
        Mesh m; TetMesh tm;
        Mesh* mesh() { return &m; }
        TetMesh* tetMesh() { return &tm; }
        bool vertexFixed(int i) const { return m.X.v[3 * i + 2] == 0.0; }
    };

    int main() {
        Obj o;
        const int n = 2;
        int64_t V, T, F;
        xpbd_grid_counts(n, n, n, &V, &T, &F);
        o.m.X.v.resize(3 * V); o.tm.E.v.resize(4 * T); o.m.F.v.resize(3 * F);
        xpbd_grid_mesh(n, n, n, 0.5, 0.5, 0.5, 0, o.m.X.v.data(), o.tm.E.v.data(), o.m.F.v.data());
        xpbd_gpu::GPUXPBDSolver<Obj> s(&o, 5, XPBD_RESIDUAL_EVERY_SUBSTEP);
        try {
            s.setup(1e-3, 9.81, [](int) { return xpbd_gpu::Material{3e3, 0.45, 1000.0}; });
        } catch (const xpbd_gpu::Error& e) {
            std::printf("status %d\n", e.status());
            return e.status() == XPBD_ERR_NO_DEVICE ? 0 : 1;
        }
        for (int k = 0; k < 10; k++) s.solve();
        std::vector<double> r = s.constraintResidual();
        std::printf("solved %zu residuals, z0=%g\n", r.size(), o.m.X.v[3 * (V - 1) + 2]);
        return r.size() == (size_t)(2 * T) ? 0 : 1;
    }
""")


def test_cpp_binding_compiles_links_and_runs(lib, tmp_path):
    src = tmp_path / "binding.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "binding"
    libdir = os.path.join(ROOT, "xpbd-tissue-sim_gb300", "_build")
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
           "-L", libdir, "-lxpbd_gpu", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("status 4") or r.stdout.startswith("solved")
