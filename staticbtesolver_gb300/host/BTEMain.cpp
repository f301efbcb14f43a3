// BTEMain.cpp -- BTEcmd: the reference's command-line tool (src/BTEMain.cpp:22-196)
// with the same flags (-g -m -b -d -t -p -T -I -x -y -z, long names as there),
// plus opt-in flags that leave the default behaviour unchanged:
//   --form plain|mixed|sweep   inner-solve form (default plain: FP64 BiCGSTAB as the reference GPU path)
//   --tol X              outer margin threshold (default 1e-5)
//   --inner-tol X        inner relative residual (default 1e-9)
//   --accel none|aitken|anderson, --accel-every N
//                        outer-iteration acceleration (default none: the reference's iteration)
//   --dsa                diffusion-synthetic correction after each outer iteration
//                        (diffusive problems; the margin and its stop are unchanged)
//   --tempcell FILE      write the cell temperatures as the reference's Tempcell.dat
//                        ("x/L_x y/L_y [z/L_z] T" per cell, src/StaticBTESolver.cpp:818-831)
#include <getopt.h>

#include <chrono>
#include <cstring>
#include <iostream>
#include <sstream>
#include <string>

#include "../../include/StaticBTESolver/StaticBTESolver.h"
#include "../../include/sbte.h"

extern "C" int sbte_main(int argc, char** argv) {
    static struct option longopts[] = {{"geometry", required_argument, nullptr, 'g'},
                                       {"material", required_argument, nullptr, 'm'},
                                       {"boundary", optional_argument, nullptr, 'b'},
                                       {"DM", required_argument, nullptr, 'd'},
                                       {"ntheta", required_argument, nullptr, 't'},
                                       {"nphi", required_argument, nullptr, 'p'},
                                       {"WFACTOR", optional_argument, nullptr, 'w'},
                                       {"T_ref", optional_argument, nullptr, 'T'},
                                       {"maxIter", optional_argument, nullptr, 'I'},
                                       {"L_x", optional_argument, nullptr, 'x'},
                                       {"L_y", optional_argument, nullptr, 'y'},
                                       {"L_z", optional_argument, nullptr, 'z'},
                                       {"form", required_argument, nullptr, 1001},
                                       {"tol", required_argument, nullptr, 1002},
                                       {"inner-tol", required_argument, nullptr, 1003},
                                       {"tempcell", required_argument, nullptr, 1004},
                                       {"accel", required_argument, nullptr, 1005},
                                       {"accel-every", required_argument, nullptr, 1006},
                                       {"dsa", no_argument, nullptr, 1007},
                                       {nullptr, 0, nullptr, 0}};
    std::string geo, bandfile, bcfile, tempcell;
    int accel = 0, accel_every = 8;
    bool dsa = false;
    double L_x = 0, L_y = 0, L_z = 0, T_ref = 300, tol = 1e-5, inner_tol = 1e-9;
    int DM = 3, ntheta = 4, nphi = 4, maxIter = 10000, form = 0;
    bool has_bc = false;
    optind = 1;
    int c, idx = 0;
    while ((c = getopt_long(argc, argv, "g:m:b:d:t:p:T:I:x:y:z:", longopts, &idx)) != -1) {
        switch (c) {
            case 'g': { std::stringstream ss(optarg); ss >> geo; break; }
            case 'm': bandfile = optarg; break;
            case 'b': has_bc = true; bcfile = optarg ? optarg : ""; break;
            case 'd': DM = std::stoi(optarg); break;
            case 't': ntheta = std::stoi(optarg); break;
            case 'p': nphi = std::stoi(optarg); break;
            case 'T': T_ref = std::stod(optarg); break;
            case 'I': maxIter = std::stoi(optarg); break;
            case 'x': L_x = std::stod(optarg); break;
            case 'y': L_y = std::stod(optarg); break;
            case 'z': L_z = std::stod(optarg); break;
            case 1001: form = std::string(optarg) == "mixed" ? 1 : std::string(optarg) == "sweep" ? 2 : 0; break;
            case 1002: tol = std::stod(optarg); break;
            case 1003: inner_tol = std::stod(optarg); break;
            case 1004: tempcell = optarg; break;
            case 1005: {
                const std::string a = optarg;
                accel = a == "anderson" ? 3 : a == "aitken" ? 2 : a == "none" ? 0 : -1;
                if (accel < 0) {
                    std::cerr << "--accel takes none, aitken or anderson" << std::endl;
                    return 1;
                }
                break;
            }
            case 1006: accel_every = std::stoi(optarg); break;
            case 1007: dsa = true; break;
            default: std::cerr << "Unknown option " << c << std::endl; return 1;
        }
    }
    BTEMesh* mesh = nullptr;
    const auto dot = geo.find_last_of('.');
    if (dot == std::string::npos) {
        mesh = new BTEMesh(std::stoi(geo), L_x);
    } else {
        const std::string ext = geo.substr(dot + 1);
        if (ext == "geo") {
            std::cout << "gmsh is not supported" << std::endl;
            return 1;
        } else if (ext == "mphtxt") {
            std::ifstream f(geo);
            mesh = new BTEMesh(f, L_x, L_y, L_z);
        } else {
            std::cout << "file format not supported" << std::endl;
            return 1;
        }
    }
    std::ifstream bf(bandfile);
    auto* bands = new BTEBand(bf);
    BTEBoundaryCondition* bcs = nullptr;
    if (has_bc) {
        std::ifstream cf(bcfile);
        bcs = new BTEBoundaryCondition(cf);
    } else {
        std::cerr << "Must specify boundary conditions" << std::endl;
        return 1;
    }
    auto start = std::chrono::steady_clock::now();
    int rc = 0;
    {
        StaticBTESolver solver(mesh, bcs, bands);
        solver.setParam(DM, ntheta, nphi, T_ref);
        solver.setForm(form);
        solver.setTolerance(tol);
        solver.setInnerTolerance(inner_tol);
        solver.setAccel(accel, accel_every);
        solver.setDsa(dsa);
        solver.solve(maxIter);
        rc = (solver.status() == 0 || solver.status() == 6) ? 0 : 1;
        if (rc == 0 && !tempcell.empty() && !solver.writeTempcell(tempcell)) {
            std::cerr << "cannot write " << tempcell << std::endl;
            rc = 1;
        }
    }
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - start).count();
    std::cout << "Time taken by process: " << ms << " milliseconds" << std::endl;  // src/BTEMain.cpp:185-188
    delete mesh;
    delete bcs;
    delete bands;
    return rc;
}
