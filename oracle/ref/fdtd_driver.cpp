// Runs the reference's finite-difference heat solver (FDTDSolver,
// src/omd/fdtd.cpp, single rank: FDTD_NO_MPI) on a spec read from standard
// input and prints the cell vector after every step.  Test infrastructure:
// the fixtures under tests/golden/ come from it.
//
// Spec lines (applied in order once `dim`, `symbol` and `map` are known):
//   dim NX NY NZ | symbol <symbol map> | map <one char per cell>
//   spacestep H | timestep DT
//   cell|conductivity|capacity|source <assignment string>
//   ext IDX VALUE        (E[IDX] = VALUE before every step)
//   steps N
//
// FDTDSolver::Step (fdtd.cpp:671-689) is an int function without a return,
// undefined behaviour that GCC may turn into a trap or a stray jump; the
// driver runs its single-rank body itself: sync_data(), Solve(), step++ (the
// communicate() call is empty without MPI).  Those members are not public,
// hence the class-key switch around the header.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include <omd/treader.h>
#define class struct
#include <misc/fdtd.hpp>
#undef class

int main() {
    int nx = 0, ny = 0, nz = 0;
    std::string symbol, map, line;
    FDTDSolver* s = 0;
    std::vector<std::pair<int, double> > ext;
    try {
        while (std::getline(std::cin, line)) {
            std::istringstream ss(line);
            std::string key;
            if (!(ss >> key)) continue;
            std::string rest;
            std::getline(ss, rest);
            if (!rest.empty() && rest[0] == ' ') rest.erase(0, 1);
            if (key == "dim") {
                std::istringstream d(rest);
                d >> nx >> ny >> nz;
            } else if (key == "symbol") {
                symbol = rest;
            } else if (key == "map") {
                map = rest;
                s = new FDTDSolver(nx, ny, nz, symbol.c_str(), map.c_str());
            } else if (!s) {
                std::fprintf(stderr, "dim, symbol and map come first\n");
                return 2;
            } else if (key == "spacestep") {
                s->SetSpacestep(std::atof(rest.c_str()));
            } else if (key == "timestep") {
                s->SetTimestep(std::atof(rest.c_str()));
            } else if (key == "cell") {
                s->SetCell(rest);
            } else if (key == "conductivity") {
                s->SetConductivity(rest);
            } else if (key == "capacity") {
                s->SetCapacity(rest);
            } else if (key == "source") {
                s->SetSource(rest);
            } else if (key == "ext") {
                std::istringstream e(rest);
                int i;
                double v;
                e >> i >> v;
                ext.push_back(std::make_pair(i, v));
            } else if (key == "steps") {
                int n = std::atoi(rest.c_str());
                const int dim = s->GetDim();
                std::printf("step %d", s->GetStep());
                for (int i = 0; i < dim; i++) std::printf(" %.17g", s->GetVector()[i]);
                std::printf("\n");
                for (int k = 0; k < n; k++) {
                    for (size_t q = 0; q < ext.size(); q++) s->GetExtVector()[ext[q].first] = ext[q].second;
                    s->sync_data();
                    s->Solve();
                    s->step++;
                    std::printf("step %d", s->GetStep());
                    for (int i = 0; i < dim; i++) std::printf(" %.17g", s->GetVector()[i]);
                    std::printf("\n");
                }
            } else {
                std::fprintf(stderr, "unknown key %s\n", key.c_str());
                return 2;
            }
        }
    } catch (const char* e) {
        std::printf("error %s\n", e);
        return 1;
    }
    delete s;
    return 0;
}
