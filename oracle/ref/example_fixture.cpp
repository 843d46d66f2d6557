// Test infrastructure: the system of the reference's example application
// (test/example/example.cpp:5-39: an FCC "111" platinum crystal, 30 x 20 x
// 10, at 100 K, EAM platinum, Verlet list, free boundaries, 0.2 ps), run by
// the reference's own MDIntegrator, with the states a GPU run needs to start
// from the same point written out: after FirstRun (BeforeRun) every atom's
// position and velocity and the box, after every step atoms 0 and 10 and the
// energies, and after the run every atom again.  tests/golden/make_golden.py
// turns the files into tests/golden/example_pt_fcc111.npz.
#include <cstdio>

#include <omd.h>

class ExampleSystem : public MDSystem {
    FILE* steps;

    void CreateSystem() {
        AddAtom(new FCC("111", 30, 20, 10, "platinum"))->Create()->SetTemperature(100.0)->SetName("Crystal");
    }

    void CreateGadget() {
        SetIntegrator(new MDIntegrator);
        AddForce(new TForceEAM("platinum"));
        AddModify(new VerletList);
        AddDetector(new ThermoDetector(0.02));
    }

    void SystemSetting() {
        PBoundary = NONPERIODIC;
        MaxTime = 0.2;
    }

    void dump_all(const char* name) {
        FILE* f = std::fopen(name, "w");
        for (int i = 0; i < GetNAtom(); i++) {
            const Atom& a = Atoms(i);
            std::fprintf(f, "%.17g %.17g %.17g %.17g %.17g %.17g\n", a.x, a.y, a.z, a.vx, a.vy, a.vz);
        }
        std::fclose(f);
    }

    void BeforeRun() {
        dump_all("start.txt");
        FILE* f = std::fopen("box.txt", "w");
        std::fprintf(f, "%.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", Box.x0, Box.y0, Box.z0, Box.x1, Box.y1,
                     Box.z1, Integrator->TimeStep, BasePotential);
        std::fclose(f);
        steps = std::fopen("steps.txt", "w");
    }

    // after Integrate, before the step's energies are measured (system.cpp:968-970)
    void InlineFunction() {
        const Atom &a = Atoms(0), &b = Atoms(10);
        std::fprintf(steps, "%.17g %.17g %.17g %.17g %.17g %.17g", a.x, a.y, a.z, b.x, b.y, b.z);
        double k = 0.0, p = 0.0;
        for (int i = 0; i < GetNAtom(); i++) {
            const Atom& c = Atoms(i);
            k += GetMass(i) * (c.vx * c.vx + c.vy * c.vy + c.vz * c.vz);
            p += c.potential;
        }
        std::fprintf(steps, " %.17g %.17g\n", 0.5 * k, p);
    }

    void AfterRun() {
        std::fclose(steps);
        dump_all("end.txt");
    }
};

int main(int argc, char* argv[]) {
    ExampleSystem sim;
    sim.SetArgument(argc, argv);
    sim.Run();
    return 0;
}
