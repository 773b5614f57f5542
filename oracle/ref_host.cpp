// ref_host.cpp -- the environment for the reference's own host steps of
// building and setting up an impact, and extern "C" entry points to them.
//
// TEST INFRASTRUCTURE.  The functions come from the reference sources, cut
// by oracle/build_ref.py into oracle/_ref/*.inc at build time (never
// committed); this file provides what they were written against -- the CUDA
// vector types, the globals of Code/CommonCode/commonSetup.h:24-60,
// Code/GenerateTargetImpactorCode/generateTargetImpactor.cu:36-37 and
// Code/ImpactCode/impactInitialization.cu:4-7 -- and sets those globals from
// the arguments before calling them.  Only the tests load it, to check the
// library's host steps bit for bit against the reference's own code.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <fstream>
#include <string>
using namespace std;

struct float4 { float x, y, z, w; };
struct double4 { double x, y, z, w; };
struct double3 { double x, y, z; };

#define ASSUMEZERODOUBLE 0.00000000001
double Pi = 3.141592654;
float4 *Pos, *Vel;
double UnitLength = -1.0, UnitTime = -1.0, Diameter = 1.0, MassSi = -1.0, MassFe = -1.0;
int TotalNumberOfElements, NSi1 = -1, NSi2 = -1, NFe1 = -1, NFe2 = -1;
double MassOfBody1 = -1.0, MassOfBody2 = -1.0;
float4 InitialPosition1, InitialPosition2, InitialVelocity1, InitialVelocity2;

// setupInitialConditions ends by moving its output file with system("mv ...")
// into the run folder; here the file is read where it was written instead.
static int ref_host_system(const char *) { return 0; }
#define system ref_host_system
#include "ref_generate_getters.inc"
#include "ref_generate_spin_drift.inc"
#include "ref_impact_setup.inc"
#undef system

namespace {

void set_bodies(float *pos, float *vel, const int counts[4], double mass_fe, double mass_si,
                double mass1, double mass2)
{
    Pos = reinterpret_cast<float4 *>(pos);
    Vel = reinterpret_cast<float4 *>(vel);
    NFe1 = counts[0];
    NSi1 = counts[1];
    NFe2 = counts[2];
    NSi2 = counts[3];
    TotalNumberOfElements = NFe1 + NSi1 + NFe2 + NSi2;
    MassFe = mass_fe;
    MassSi = mass_si;
    MassOfBody1 = mass1;
    MassOfBody2 = mass2;
}

}  // namespace

// spinBody(body, spin) on pos / vel in [Fe1, Si1, Fe2, Si2] order;
// counts = NFe1, NSi1, NFe2, NSi2; spin = axis xyz and rate w.
extern "C" void giref_host_spin(float *pos, float *vel, const int counts[4], double mass_fe,
                                double mass_si, double mass1, double mass2, int body,
                                const float spin[4])
{
    set_bodies(pos, vel, counts, mass_fe, mass_si, mass1, mass2);
    float4 s = {spin[0], spin[1], spin[2], spin[3]};
    spinBody(body, s);
}

// zeroOutTargetImpactorDrift() on pos / vel.
extern "C" void giref_host_zero_drift(float *pos, float *vel, const int counts[4], double mass_fe,
                                      double mass_si, double mass1, double mass2)
{
    set_bodies(pos, vel, counts, mass_fe, mass_si, mass1, mass2);
    zeroOutTargetImpactorDrift();
}

// readImpactSetupParameters() + setupInitialConditions() run in work_dir,
// which must hold the reference's layout: setupImpactInitialization and
// TargetImpactorInformation/targetImpactorInitialPosVel two levels above
// work_dir.  The initial frame they write (work_dir/impactPosVel) is read
// back into pos_out / vel_out.  Returns 0, or -1 when a file cannot be used.
extern "C" int giref_host_impact_setup(const char *work_dir, const int counts[4],
                                       double unit_length, double unit_time, float *pos_out,
                                       float *vel_out)
{
    char prev[4096];
    if (!getcwd(prev, sizeof prev) || chdir(work_dir) != 0) return -1;
    NFe1 = counts[0];
    NSi1 = counts[1];
    NFe2 = counts[2];
    NSi2 = counts[3];
    TotalNumberOfElements = NFe1 + NSi1 + NFe2 + NSi2;
    UnitLength = unit_length;
    UnitTime = unit_time;
    readImpactSetupParameters();
    setupInitialConditions();
    int status = -1;
    FILE *f = fopen("impactPosVel", "rb");
    if (f) {
        float t = 0.0f;
        const size_t n = (size_t)TotalNumberOfElements;
        if (fread(&t, sizeof t, 1, f) == 1 && fread(pos_out, 16, n, f) == n &&
            fread(vel_out, 16, n, f) == n)
            status = 0;
        fclose(f);
    }
    free(Pos);
    free(Vel);
    Pos = Vel = nullptr;
    if (chdir(prev) != 0) return -1;
    return status;
}
