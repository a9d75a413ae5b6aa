// ref_harness.cpp -- drives the reference SOLVEiT force methods headlessly.
//
// TEST INFRASTRUCTURE ONLY.  Linked against the reference sources as they
// lie in the reference tree (see oracle/Makefile, target `ref`); the resulting binary
// lives in oracle/_ref/ and is used to generate golden fixtures and to pin
// the oracle restatement.  It fills a ChargedParticles instance by hand (the
// shipped driver needs data files the reference does not ship) and calls the
// reference's own updateAcceleration() / propagate*New() methods.
//
// usage: ref_harness <mode> <in.bin> <out.bin> [key=value ...]
//   modes: direct | bh | fmm | dkd | grid | outliers
//          (outliers mode: int32 count, int32 outlierCheck[n] of
//           DomainBoundsFunction::isOutlier)
//   keys : threads, sym (0 none, 1 rotational, 2 translational), levels,
//          axes (e.g. 110), dom (domain size x,y,z in metres), theta, p,
//          maxlevel, steps, dt, ez;
//          dkd only: crash (1 extractor grid), cz, cw, cr (z_distance,
//          z_width, r_distance), bc (BoundaryConditionOptions 0..3), bx, by,
//          bz, br (spatial limits), bt (temporal limit), events (1: append the
//          events file);
//          efield and dkd: fdir (folder, with its trailing /), fnodes, ftris
//          (the Fields / Triangles files in the reference's CSV format), r0, e0:
//          a singleEmitter background field (dkd: replaces ez)
//   mode efield: InterpolationScheme::Efield at each particle, float e[3n]
//   mode run: the reference's own integrator, LeapfrogDKD::runSimulation, or
//          with subs=dt,bc,bx,by,bz,br,bt;... LeapfrogDKDSubsteps with
//          setSubstepTimes (direct force); keys steps, dt, crash / bc keys as
//          dkd; out.bin as dkd, then int32 bytes and the snapshot file
//          (SaveDataOptions::newOriginal) written at the start and the end;
//          interval=k: saveData and the energy records every k steps;
//          energy=init,steps with edir=<folder/>: Integrator::toggleEnergy
//          (its file goes to edir), out.bin then ends with int32 records and
//          the energy file (six floats per record)
// in.bin : int32 n, float pos4[4n], float vel4[4n], float acc4[4n], float tinj[n]
// out.bin: float pos4[4n], float vel4[4n], float acc4[4n]
//          (dkd with events=1: then int32 count, count 40-byte event records
//          as ChargedParticles::writeToEventsFile wrote them)
//          (grid mode: int32 count, int32 points[3*count] in the Grid's order)
// stderr : the single-evaluation modes (direct, bh, fmm) print
//          update_s=<wall seconds of updateAcceleration()> threads=<t> n=<n>
#include "force_calculation_methods.h"
#include "integration_schemes.h"

#include <dirent.h>

#include <chrono>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

static std::map<std::string, std::string> parse_kv(int argc, char **argv, int first) {
    std::map<std::string, std::string> kv;
    for (int i = first; i < argc; i++) {
        const char *eq = std::strchr(argv[i], '=');
        if (!eq) continue;
        kv[std::string(argv[i], eq - argv[i])] = std::string(eq + 1);
    }
    return kv;
}

// a scratch file beside out.bin (the caller's directory), read back and removed
static FILE *scratch_file(const char *out_path, const char *name) {
    std::string dir(out_path);
    const size_t slash = dir.find_last_of('/');
    dir = slash == std::string::npos ? std::string() : dir.substr(0, slash + 1);
    const std::string path = dir + name;
    FILE *f = std::fopen(path.c_str(), "w+b");
    if (f) std::remove(path.c_str());  // the open handle keeps it until closed
    return f;
}

static double getd(std::map<std::string, std::string> &kv, const char *k, double d) {
    auto it = kv.find(k);
    return it == kv.end() ? d : std::atof(it->second.c_str());
}

int main(int argc, char **argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s mode in.bin out.bin [k=v ...]\n", argv[0]);
        return 2;
    }
    std::string mode = argv[1];
    auto kv = parse_kv(argc, argv, 4);
    const bool field = kv.count("fdir") > 0;
    const int threads = (int)getd(kv, "threads", 1);
    const int sym = (int)getd(kv, "sym", 0);
    const int levels = (int)getd(kv, "levels", 2);
    std::string axes_s = kv.count("axes") ? kv["axes"] : "110";
    vec3<int> axes(axes_s[0] - '0', axes_s[1] - '0', axes_s[2] - '0');

    if (mode == "grid") {
        int box_length = 1;
        for (int l = 0; l < levels; l++) box_length *= 3;
        Grid grid(box_length, axes);
        FILE *fo = std::fopen(argv[3], "wb");
        if (!fo) return 3;
        int32_t cnt = grid.numLattice;
        std::fwrite(&cnt, 4, 1, fo);
        for (int i = 0; i < grid.numLattice; i++) {
            int32_t p[3] = {grid.lattice[i].point.x, grid.lattice[i].point.y, grid.lattice[i].point.z};
            std::fwrite(p, 4, 3, fo);
        }
        std::fclose(fo);
        return 0;
    }

    FILE *fi = std::fopen(argv[2], "rb");
    if (!fi) return 3;
    int32_t n = 0;
    if (std::fread(&n, 4, 1, fi) != 1 || n <= 0) return 4;
    ParticleSystem ps;
    ChargedParticles &cp = ps.chargedParticles;
    cp.allocateMemory(n);
    bool ok = std::fread(cp.position, 16, n, fi) == (size_t)n &&
              std::fread(cp.velocity, 16, n, fi) == (size_t)n &&
              std::fread(cp.acceleration, 16, n, fi) == (size_t)n &&
              std::fread(cp.timeInjected, 4, n, fi) == (size_t)n;
    std::fclose(fi);
    if (!ok) return 4;
    for (int i = 0; i < n; i++) {
        cp.Efield1[i] = 0.0f;
        cp.Efield2[i] = 0.0f;
    }
    cp.firstParticle = 0;
    cp.lastParticle = n;
    if (field) {
        // ParticleSystem::initializeBackgroundEField (particles.cpp:452-463)
        ps.params.r0 = (float)getd(kv, "r0", 1.0);
        ps.params.E0 = (float)getd(kv, "e0", 1.0);
        ps.initializeBackgroundEField(BackgroundEfield::singleEmitter, kv["fdir"].c_str(), kv["fnodes"].c_str(),
                                      kv["ftris"].c_str());
    }

    if (mode == "efield") {
        FILE *fo = std::fopen(argv[3], "wb");
        if (!fo) return 3;
        for (int i = 0; i < n; i++) {
            vec3<float> e = ps.interpScheme.Efield(cp.position[i].x, cp.position[i].y, cp.position[i].z);
            const float v[3] = {e.x, e.y, e.z};
            std::fwrite(v, 4, 3, fo);
        }
        std::fclose(fo);
        std::fflush(nullptr);
        std::_Exit(0);
    }

    if (mode == "outliers") {
        std::vector<int> check(n, 0);
        int count = 0;
        DomainBoundsFunction::isOutlier(cp, check.data(), count);
        FILE *fo = std::fopen(argv[3], "wb");
        if (!fo) return 3;
        const int32_t cnt = count;
        std::fwrite(&cnt, 4, 1, fo);
        for (int i = 0; i < n; i++) {
            const int32_t v = check[i];
            std::fwrite(&v, 4, 1, fo);
        }
        std::fclose(fo);
        std::fflush(nullptr);
        std::_Exit(0);
    }

    ps.params.numThreads = threads;
    ps.params.symType = sym == 1 ? SymmetryType::rotational
                      : sym == 2 ? SymmetryType::translational : SymmetryType::none;
    ps.params.symmetryAxes = axes;
    ps.params.numSymmetryLevels = levels;
    std::string dom = kv.count("dom") ? kv["dom"] : "2e-6,2e-6,0";
    float d[3] = {0, 0, 0};
    std::sscanf(dom.c_str(), "%f,%f,%f", &d[0], &d[1], &d[2]);
    ps.params.domainSize = vec3<float>(d[0], d[1], d[2]);

    int box_length = 1;
    for (int l = 0; l < levels; l++) box_length *= 3;
    Grid grid(box_length, axes);

    MultipoleMethodConstants mc;
    MultipoleMethodVariables mv;
    ForceCalculationMethod *fm = nullptr;
    DirectForceCalculation *df = nullptr;
    BarnesHutForceCalculation *bh = nullptr;
    MultipoleMethodForceCalculation *fmm = nullptr;
    if (mode == "direct" || mode == "dkd" || mode == "run") {
        df = new DirectForceCalculation(&ps);
        fm = df;
    } else if (mode == "bh") {
        bh = new BarnesHutForceCalculation(&ps);
        bh->setTheta((float)getd(kv, "theta", 0.5));
        fm = bh;
    } else if (mode == "fmm") {
        fmm = new MultipoleMethodForceCalculation(&ps, &mc, &mv, FmmType::fmm);
        fmm->setNumExpansions((int)getd(kv, "p", 8));
        if (kv.count("maxlevel")) fmm->setMaxLevel((int)getd(kv, "maxlevel", 0));
        fm = fmm;
    } else {
        std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
        return 2;
    }
    fm->setFirstParticle(0);
    fm->setLastParticle(n);
    fm->setGrid(&grid);

    FILE *events = nullptr;
    FILE *snap = nullptr;
    if (mode == "run") {
        const int steps = (int)getd(kv, "steps", 1);
        ps.params.timeStep = (float)getd(kv, "dt", 1e-13);
        ps.params.numIters = steps;
        ps.params.interval = (int)getd(kv, "interval", steps);  // saveData every interval (constantRate)
        ps.params.timerInfo = TimerOptions::off;
        ps.params.saveDataToggle = SaveDataOptions::newOriginal;
        snap = scratch_file(argv[3], "snapshot.tmp");
        events = scratch_file(argv[3], "events.tmp");
        if (!snap || !events) return 3;
        static FILE *files[1];
        files[0] = snap;
        ps.params.saveDataFiles = files;
        ps.params.numSaveDataFiles = 1;
        ps.params.eventsFile = events;
        CrashParameters &cr = ps.params.crashParameters;
        cr.crashOptions = getd(kv, "crash", 0) != 0 ? CrashConditionOptions::extractorGrid
                                                     : CrashConditionOptions::none;
        cr.z_distance = (float)getd(kv, "cz", 0.0);
        cr.z_width = (float)getd(kv, "cw", 0.0);
        cr.r_distance = (float)getd(kv, "cr", 0.0);
        BoundaryConditionParameters &bc = ps.params.boundaryConditions;
        const int bck = (int)getd(kv, "bc", 0);
        bc.boundaryConditionType = bck == 1 ? BoundaryConditionOptions::space
                                 : bck == 2 ? BoundaryConditionOptions::time
                                 : bck == 3 ? BoundaryConditionOptions::space_and_time
                                            : BoundaryConditionOptions::none;
        bc.spatialBoundaryConditions = vec4<float>((float)getd(kv, "bx", 0.0), (float)getd(kv, "by", 0.0),
                                                   (float)getd(kv, "bz", 0.0), (float)getd(kv, "br", 0.0));
        bc.temporalBoundaryCondition = (float)getd(kv, "bt", 0.0);
        if (kv.count("subs")) {
            // "dt,bc,bx,by,bz,br,bt;..." -> setSubstepTimes(times, bcs, size)
            std::vector<float> times;
            std::vector<BoundaryConditionParameters> bcs;
            std::string list = kv["subs"];
            size_t pos = 0;
            while (pos < list.size()) {
                size_t end = list.find(';', pos);
                if (end == std::string::npos) end = list.size();
                float v[7] = {0, 0, 0, 0, 0, 0, 0};
                std::sscanf(list.substr(pos, end - pos).c_str(), "%f,%f,%f,%f,%f,%f,%f", &v[0], &v[1], &v[2], &v[3],
                            &v[4], &v[5], &v[6]);
                BoundaryConditionParameters b;
                const int k = (int)v[1];
                b.boundaryConditionType = k == 1 ? BoundaryConditionOptions::space
                                        : k == 2 ? BoundaryConditionOptions::time
                                        : k == 3 ? BoundaryConditionOptions::space_and_time
                                                 : BoundaryConditionOptions::none;
                b.spatialBoundaryConditions = vec4<float>(v[2], v[3], v[4], v[5]);
                b.temporalBoundaryCondition = v[6];
                times.push_back(v[0]);
                bcs.push_back(b);
                pos = end + 1;
            }
            LeapfrogDKDSubsteps leap(ps, *fm);
            leap.setSubstepTimes(times.data(), bcs.data(), (int)times.size());
            leap.runSimulation();
        } else {
            LeapfrogDKD leap(ps, *fm);
            if (kv.count("energy")) {
                int init = 0, each = 0;
                std::sscanf(kv["energy"].c_str(), "%d,%d", &init, &each);
                leap.toggleEnergy(1, init, each, kv["edir"].c_str());
            }
            leap.runSimulation();
        }
    } else if (mode == "dkd") {
        // LeapfrogDKD::runSimulation step structure (integration_schemes.cpp:
        // 867-888) with driftNew's injection window (:705-723) on the
        // reference's own methods: findMostRecentInjected, ParticleSystem::
        // propagatePositionNew (drift with the crash test, symmetry folding,
        // boundary conditions), resetFirstChargedParticle and
        // propagateVelocityNew.  The uniform background field is added as
        // computeBackgroundAcceleration adds the interpolated one
        // (particles.cpp:496-520), over the same window.
        const int steps = (int)getd(kv, "steps", 1);
        const float dt = (float)getd(kv, "dt", 1e-13);
        const float ez = (float)getd(kv, "ez", 0.0);
        CrashParameters &cr = ps.params.crashParameters;
        cr.crashOptions = getd(kv, "crash", 0) != 0 ? CrashConditionOptions::extractorGrid
                                                     : CrashConditionOptions::none;
        cr.z_distance = (float)getd(kv, "cz", 0.0);
        cr.z_width = (float)getd(kv, "cw", 0.0);
        cr.r_distance = (float)getd(kv, "cr", 0.0);
        BoundaryConditionParameters &bc = ps.params.boundaryConditions;
        const int bck = (int)getd(kv, "bc", 0);
        bc.boundaryConditionType = bck == 1 ? BoundaryConditionOptions::space
                                 : bck == 2 ? BoundaryConditionOptions::time
                                 : bck == 3 ? BoundaryConditionOptions::space_and_time
                                            : BoundaryConditionOptions::none;
        bc.spatialBoundaryConditions = vec4<float>((float)getd(kv, "bx", 0.0), (float)getd(kv, "by", 0.0),
                                                   (float)getd(kv, "bz", 0.0), (float)getd(kv, "br", 0.0));
        bc.temporalBoundaryCondition = (float)getd(kv, "bt", 0.0);
        events = scratch_file(argv[3], "events.tmp");
        if (!events) return 3;
        ps.params.eventsFile = events;
        const float inbound = 1.0f;
        const double factor = PhysicalConstant::ELEM_CHARGE / PhysicalConstant::AMU;
        auto drift_new = [&](float tstart, float h) {
            const int last = cp.findMostRecentInjected(tstart + h) + 1;
            cp.lastParticle = last;
            fm->setLastParticle(last);
            ps.propagatePositionNew(tstart, h);
            ps.resetFirstChargedParticle();
            fm->setFirstParticle(cp.firstParticle);
        };
        cp.lastParticle = 0;
        for (int it = 1; it <= steps; it++) {
            float tpos = dt * (it - 1);
            float tvel = dt * (it - 1);
            drift_new(tpos, dt / 2);
            tpos += dt / 2;
            cp.zeroAcceleration();
            fm->updateAcceleration();
            if (field) {
                ps.computeBackgroundAcceleration();
            } else {
                for (int i = cp.firstParticle; i < cp.lastParticle; i++) {
                    if (cp.acceleration[i].w != inbound) continue;
                    float efactor = factor * cp.position[i].w / cp.getMass(i);
                    vec3<float> e(0.0f, 0.0f, ez);
                    e *= efactor;
                    cp.acceleration[i].x += e.x;
                    cp.acceleration[i].y += e.y;
                    cp.acceleration[i].z += e.z;
                }
            }
            ps.propagateVelocityNew(tvel, dt);
            drift_new(tpos, dt / 2);
        }
    } else {
        const auto t0 = std::chrono::steady_clock::now();
        fm->updateAcceleration();
        const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::fprintf(stderr, "update_s=%.6f threads=%d n=%d\n", sec, threads, n);
    }

    FILE *fo = std::fopen(argv[3], "wb");
    if (!fo) return 3;
    std::fwrite(cp.position, 16, n, fo);
    std::fwrite(cp.velocity, 16, n, fo);
    std::fwrite(cp.acceleration, 16, n, fo);
    if (snap) {
        std::fflush(snap);
        const long bytes = std::ftell(snap);
        const int32_t cnt = (int32_t)bytes;
        std::fwrite(&cnt, 4, 1, fo);
        std::rewind(snap);
        std::vector<char> buf((size_t)bytes);
        if (bytes > 0 && std::fread(buf.data(), 1, (size_t)bytes, snap) != (size_t)bytes) return 5;
        if (bytes > 0) std::fwrite(buf.data(), 1, (size_t)bytes, fo);
    }
    if (events && getd(kv, "events", 0) != 0) {
        std::fflush(events);
        const long bytes = std::ftell(events);
        const int32_t cnt = (int32_t)(bytes / 40);
        std::fwrite(&cnt, 4, 1, fo);
        std::rewind(events);
        std::vector<char> buf((size_t)bytes);
        if (bytes > 0 && std::fread(buf.data(), 1, (size_t)bytes, events) != (size_t)bytes) return 5;
        if (bytes > 0) std::fwrite(buf.data(), 1, (size_t)bytes, fo);
    }
    if (mode == "run" && kv.count("energy")) {
        // the one file toggleEnergy created in edir (closed with the integrator)
        std::string path;
        if (DIR *d = opendir(kv["edir"].c_str())) {
            while (dirent *e = readdir(d))
                if (std::strncmp(e->d_name, "energy_", 7) == 0) path = kv["edir"] + e->d_name;
            closedir(d);
        }
        std::vector<char> buf;
        if (FILE *fe = path.empty() ? nullptr : std::fopen(path.c_str(), "rb")) {
            char tmp[4096];
            size_t got;
            while ((got = std::fread(tmp, 1, sizeof tmp, fe)) > 0) buf.insert(buf.end(), tmp, tmp + got);
            std::fclose(fe);
        }
        const int32_t cnt = (int32_t)(buf.size() / 24);
        std::fwrite(&cnt, 4, 1, fo);
        if (!buf.empty()) std::fwrite(buf.data(), 1, (size_t)cnt * 24, fo);
    }
    std::fclose(fo);
    // SimulationParameters' destructor releases members the headless set-up
    // never initialised (file handles, storage arrays); leave without running
    // destructors once the outputs are on disk.
    std::fflush(nullptr);
    std::_Exit(0);
}
