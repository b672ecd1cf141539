"""The C++ host of the YAML-configured Simulation (include/xpbd_simulation.hpp)
against the Python host (xpbd-tissue-sim_gb300/simulation.py, yaml_lite.py,
msh.py), which the other tests check against the reference's behaviour:
the same parsed configs (our scenes and, where the reference checkout is on
this machine, every one of its config files), the same gmsh reading and mesh
placement, and on a GPU the same trajectory."""
import json
import math
import os
import subprocess
import textwrap

import numpy as np
import pytest

import msh
import simulation as S
import xpbd_gb300 as G
import yaml_lite as Y
from conftest import reference_dir

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = textwrap.dedent(r"""
    #include <cstdio>
    #include <cstring>
    #include <string>
    #include "xpbd_simulation.hpp"
    using namespace xpbd_sim;

    static void vec(const char* k, const Vec3& v, bool comma = true) {
        std::printf("\"%s\": [%.17g, %.17g, %.17g]%s", k, v[0], v[1], v[2], comma ? ", " : "");
    }
    static void dump_config(const SimulationConfig& c) {
        std::printf("{\"name\": \"%s\", \"time_step\": %.17g, \"end_time\": %.17g, \"g_accel\": %.17g, "
                    "\"collision_rate\": %.17g, \"sim_mode\": \"%s\", \"visualization\": \"%s\", \"materials\": [",
                    c.name.c_str(), c.time_step, c.end_time, c.g_accel, c.collision_rate, c.sim_mode.c_str(),
                    c.visualization.c_str());
        for (size_t i = 0; i < c.materials.size(); i++) {
            const auto& m = c.materials[i];
            std::printf("%s{\"name\": \"%s\", \"density\": %.17g, \"E\": %.17g, \"nu\": %.17g, \"mu_s\": %.17g, "
                        "\"mu_k\": %.17g}", i ? ", " : "", m.name.c_str(), m.density, m.E, m.nu, m.mu_s, m.mu_k);
        }
        std::printf("], \"objects\": [");
        for (size_t i = 0; i < c.objects.size(); i++) {
            const auto& o = c.objects[i];
            std::printf("%s{\"type\": %d, \"name\": \"%s\", \"collisions\": %d, \"graphics_only\": %d, ", i ? ", " : "",
                        (int)o.type, o.name.c_str(), (int)o.collisions, (int)o.graphics_only);
            vec("position", o.position); vec("velocity", o.velocity); vec("rotation", o.rotation);
            if (o.rigid()) {
                std::printf("\"radius\": %.17g, \"density\": %.17g, \"fixed\": %d, \"height\": %.17g, ", o.radius,
                            o.density, (int)o.fixed, o.height);
                vec("size", o.size); vec("angular_velocity", o.angular_velocity, false);
            } else {
                std::printf("\"filename\": \"%s\", \"num_solver_iters\": %d, \"num_local_collision_iters\": %d, "
                            "\"solver_type\": %d, \"constraint_type\": %d, \"residual_policy\": %d, "
                            "\"self_collisions\": %d, \"max_size\": %.17g, \"damping_multiplier\": %.17g, "
                            "\"adjust_damping_to_material\": %d, \"materials\": [",
                            o.filename.c_str(), o.num_solver_iters, o.num_local_collision_iters, o.solver_type,
                            o.constraint_type, o.residual_policy, (int)o.self_collisions, o.max_size,
                            o.damping_multiplier, (int)o.adjust_damping_to_material);
                for (size_t k = 0; k < o.materials.size(); k++) std::printf("%s\"%s\"", k ? ", " : "", o.materials[k].c_str());
                std::printf("]");
            }
            std::printf("}");
        }
        std::printf("]}\n");
    }
    static void write(const char* path, const std::vector<double>& a) {
        FILE* f = std::fopen(path, "wb");
        std::fwrite(a.data(), sizeof(double), a.size(), f);
        std::fclose(f);
    }

    int main(int argc, char** argv) {
        try {
            const std::string mode = argv[1];
            if (mode == "cfg") {
                dump_config(parse_config(load_yaml(argv[2])));
            } else if (mode == "place") {  // msh px py pz rx ry rz max_size out
                TetMesh m = read_msh(argv[2]);
                const Vec3 p{std::atof(argv[3]), std::atof(argv[4]), std::atof(argv[5])};
                const Vec3 r{std::atof(argv[6]), std::atof(argv[7]), std::atof(argv[8])};
                place(m, p, r, std::atof(argv[9]), nullptr);
                write(argv[10], m.X);
                std::printf("%lld %lld %lld\n", (long long)m.V(), (long long)m.T(), (long long)m.F());
            } else if (mode == "run") {  // yaml steps out
                Simulation sim(argv[2]);
                sim.setup();
                const int n = sim.update(std::atoi(argv[3]));
                std::vector<double> all;
                for (auto& o : sim.objects()) {
                    const auto x = sim.positions(o.cfg.name);
                    all.insert(all.end(), x.begin(), x.end());
                }
                write(argv[4], all);
                std::printf("steps %d time %.17g\n", n, sim.time());
            }
        } catch (const std::exception& e) {
            std::printf("error: %s\n", e.what());
            return 3;
        }
        return 0;
    }
""")


@pytest.fixture(scope="module")
def exe(lib, tmp_path_factory):
    d = tmp_path_factory.mktemp("cppsim")
    src = d / "sim.cpp"
    src.write_text(PROGRAM)
    out = d / "sim"
    libdir = os.path.join(ROOT, "xpbd-tissue-sim_gb300", "_build")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                        str(out), "-L", libdir, "-lxpbd_gpu", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(out)


def _py_config(path):
    c = S.load_config(path)[0]
    kinds = {S.RigidBoxConfig: 3, S.RigidCylinderConfig: 4, S.RigidSphereConfig: 2}
    objs = []
    for o in c.objects:
        if isinstance(o, S.RigidSphereConfig):
            t = kinds[type(o)]
            d = {"type": t, "name": o.name, "collisions": int(o.collisions), "graphics_only": int(o.graphics_only),
                 "position": list(o.position), "velocity": list(o.velocity), "rotation": list(o.rotation),
                 "radius": o.radius, "density": o.density, "fixed": int(o.fixed),
                 "height": getattr(o, "height", 1.0), "size": list(getattr(o, "size", [1.0, 1.0, 1.0])),
                 "angular_velocity": list(o.angular_velocity)}
        else:
            d = {"type": 1 if o.first_order else 0, "name": o.name, "collisions": int(o.collisions),
                 "graphics_only": int(o.graphics_only), "position": list(o.position), "velocity": list(o.velocity),
                 "rotation": list(o.rotation), "filename": o.filename, "num_solver_iters": o.num_solver_iters,
                 "num_local_collision_iters": o.num_local_collision_iters, "solver_type": o.solver_type,
                 "constraint_type": o.constraint_type, "residual_policy": o.residual_policy,
                 "self_collisions": int(o.self_collisions),
                 "max_size": -1.0 if o.max_size is None else o.max_size,
                 "damping_multiplier": o.damping_multiplier,
                 "adjust_damping_to_material": int(o.adjust_damping_to_material), "materials": list(o.materials)}
        objs.append(d)
    return {"name": c.name, "time_step": c.time_step, "end_time": c.end_time, "g_accel": c.g_accel,
            "collision_rate": c.collision_rate, "sim_mode": c.sim_mode, "visualization": c.visualization,
            "materials": [{"name": m.name, "density": m.density, "E": m.E, "nu": m.nu, "mu_s": m.mu_s,
                           "mu_k": m.mu_k} for m in c.materials], "objects": objs}


def _cpp_config(exe, path):
    r = subprocess.run([exe, "cfg", path], capture_output=True, text=True, timeout=60)
    assert r.returncode in (0, 3), r.stderr
    if r.stdout.startswith("error:"):
        return r.stdout.strip()
    return json.loads(r.stdout)


def test_cpp_config_reader_matches_python(exe, tmp_path):
    from test_simulation_config import CONFIG
    p = tmp_path / "scene.yaml"
    p.write_text(CONFIG)
    assert _cpp_config(exe, str(p)) == _py_config(str(p))


def test_cpp_config_reader_matches_python_on_reference_configs(exe):
    ref = reference_dir()
    if not ref or not os.path.isdir(os.path.join(ref, "config")):
        pytest.skip("reference configs not present")
    import glob
    files = sorted(glob.glob(os.path.join(ref, "config", "**", "*.yaml"), recursive=True))
    assert files
    compared = 0
    for f in files:
        try:
            py = _py_config(f)
        except (NotImplementedError, ValueError) as e:
            out = _cpp_config(exe, f)
            assert isinstance(out, str) and out.startswith("error:"), (f, e, out)
            continue
        assert _cpp_config(exe, f) == py, f
        compared += 1
    assert compared > 0


def test_cpp_msh_reader_and_placement_match_python(exe, tmp_path):
    X, tets, faces = G.grid_mesh(3, 4, 2, 0.1)
    X = X + np.random.default_rng(3).uniform(-0.01, 0.01, X.shape)
    path = str(tmp_path / "m.msh")
    msh.write_msh(path, X, tets, faces)
    out = str(tmp_path / "x.bin")
    args = [0.1, -0.2, 0.5, 10.0, 20.0, 30.0, 0.5]
    r = subprocess.run([exe, "place", path] + [repr(a) for a in args] + [out], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.split() == [str(X.shape[0]), str(tets.shape[0]), str(faces.shape[0])]
    xc = np.fromfile(out, np.float64).reshape(-1, 3)
    Xr, tr, fr = msh.read_msh(path)
    xp = msh.place(Xr, fr, args[:3], args[3:6], args[6], None)
    np.testing.assert_allclose(xc, xp, rtol=0, atol=1e-14)


@pytest.mark.gpu
def test_cpp_simulation_runs_the_same_trajectory_as_python(exe, tmp_path):
    from test_gpu_simulation import _scene
    cfg, X, tets, faces = _scene(tmp_path, end=0.04)
    out = str(tmp_path / "x.bin")
    r = subprocess.run([exe, "run", cfg, "40", out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("steps 40"), r.stdout + r.stderr
    xc = np.fromfile(out, np.float64).reshape(-1, 3)
    with S.Simulation(cfg) as sim:
        sim.setup()
        assert sim.update(max_steps=40) == 40
        xp = sim.objects["Cube"].positions()
    moved = np.abs(xp - msh.place(X, faces, [0.1, 0, 0.5], [0, 0, 30], 0.5, None)).max()
    assert moved > 1e-3
    # the same inputs up to double rounding in placement: identical device work
    np.testing.assert_allclose(xc, xp, rtol=0, atol=1e-6)
