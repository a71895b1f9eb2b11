// cpmp_run.cpp -- command-line driver with the reference's host loop.
//
// Replaces main() of the reference (FluidCuda.cu:1245-1312) on top of the C
// ABI: one initialisation and one droplet, then a BasePt sweep that carries
// the state from one wall potential to the next without re-initialising
// (:1262-1264), the ShowStep/SaveStep cadence (:1296-1301), the stdout table
// of ShowData (:1658-1732) and the contact-angle file of SaveContactAngle
// (:1735-1771), and the x-z density slice ContactAngle writes (:580-589).
// The output streams are written with the same iostream
// manipulators in the same order, so the sticky stream state of the
// reference (std::fixed and the last precision carry over from one table
// to the next header) is reproduced as well.
//
// Options (defaults are the reference's Initialize(), FluidCuda.cu:119-163):
//   --dx/--dy/--dz N            grid (the reference's is compile-time)
//   --model NAME|ID             CP_VDW CP_PRW CP_PRM CP_RKE CP_RKS CP_CSE
//   --tr --k --ka --k1 --k2 --tau --eos-a --eos-b --eos-omega X
//   --radius R --width W        droplet; placed as the reference places it
//   --centre X,Y,Z              explicit droplet centre instead
//   --lap 5|7  --simple-bc      Laplacian order, single-layer wall rule
//   --storage f64|f32|f16|bf16  --scheme plain|fused  --device N
//   --cocurve-dir DIR           CoCurve_<EOS>_2.txt tables (default: Maxwell)
//   --allstep N --showstep N --savestep N
//   --basept-from A --basept-to B --basept-step S
//                               the reference's sweep: for (v = A; v <= B; v += S)
//   --basept v1,v2,...          an explicit list instead
//   --reinit                    re-initialise the droplet for every BasePt
//   --out-dir DIR               where the contact-angle file goes (default data)
//   --ca-header                 write the column header of the contact-angle
//                               file (the reference's condition for it,
//                               No == 0 && NowStep == 0, never holds at the
//                               only call site, NowStep == AllStep)
//   --dry-run                   print the parameter block, the sweep values and
//                               the contact-angle file name; no GPU is used
#include <sys/stat.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "cpmp.h"

using namespace std;

namespace {

struct Run {
    cpmp_params p;
    double radius = 60, width = 10;
    bool has_centre = false;
    double cx = 0, cy = 0, cz = 0;
    long allstep = 100L * 10000, showstep = 10000, savestep = 10000;
    double bp_from = -0.08, bp_to = -0.015, bp_step = 0.005;
    vector<double> bp_list;
    bool reinit = false, ca_header = false, dry = false;
    string out_dir = "data", cocurve;
};

const char *model_name(int m)
{
    switch (m) {
    case CPMP_MP_CPVDW: return "CP_VDW";
    case CPMP_MP_CPPRW: return "CP_PRW";
    case CPMP_MP_CPPRM: return "CP_PRM";
    case CPMP_MP_CPRKE: return "CP_RKE";
    case CPMP_MP_CPRKS: return "CP_RKS";
    case CPMP_MP_CPCSE: return "CP_CSE";
    }
    return "Unknown";
}

int parse_model(const string &s)
{
    for (int m = CPMP_MP_CPVDW; m <= CPMP_MP_CPCSE; ++m)
        if (s == model_name(m)) return m;
    return atoi(s.c_str());
}

[[noreturn]] void usage(const char *msg)
{
    cerr << "cpmp_run: " << msg << "\n(see the option list at the top of cpmp_run.cpp)" << endl;
    exit(2);
}

Run parse(int argc, char **argv)
{
    Run r;
    cpmp_params_default(&r.p);
    for (int a = 1; a < argc; ++a) {
        string k = argv[a];
        auto val = [&]() -> string {
            if (a + 1 >= argc) usage(("missing value for " + k).c_str());
            return argv[++a];
        };
        auto num = [&]() { return atof(val().c_str()); };
        if (k == "--dx") r.p.dx = (int)num();
        else if (k == "--dy") r.p.dy = (int)num();
        else if (k == "--dz") r.p.dz = (int)num();
        else if (k == "--model") r.p.model = parse_model(val());
        else if (k == "--tr") r.p.tr = num();
        else if (k == "--k") r.p.k = num();
        else if (k == "--ka") r.p.ka = num();
        else if (k == "--k1") r.p.k1 = num();
        else if (k == "--k2") r.p.k2 = num();
        else if (k == "--tau") r.p.tau = num();
        else if (k == "--eos-a") r.p.eos_a = num();
        else if (k == "--eos-b") r.p.eos_b = num();
        else if (k == "--eos-omega") r.p.eos_omega = num();
        else if (k == "--radius") r.radius = num();
        else if (k == "--width") r.width = num();
        else if (k == "--centre") {
            if (sscanf(val().c_str(), "%lf,%lf,%lf", &r.cx, &r.cy, &r.cz) != 3) usage("--centre wants X,Y,Z");
            r.has_centre = true;
        } else if (k == "--lap") r.p.lap_order = (int)num();
        else if (k == "--simple-bc") r.p.complex_bc = 0;
        else if (k == "--storage") {
            const string s = val();
            r.p.storage = s == "f64" ? CPMP_STORE_F64 : s == "f32" ? CPMP_STORE_F32 : s == "f16" ? CPMP_STORE_F16
                        : s == "bf16" ? CPMP_STORE_BF16 : (usage("storage is f64, f32, f16 or bf16"), 0);
        } else if (k == "--scheme") {
            const string s = val();
            r.p.scheme = s == "plain" ? CPMP_SCHEME_PLAIN : s == "fused" ? CPMP_SCHEME_FUSED
                       : (usage("scheme is plain or fused"), 0);
        } else if (k == "--device") r.p.device = (int)num();
        else if (k == "--cocurve-dir") r.cocurve = val();
        else if (k == "--allstep") r.allstep = atol(val().c_str());
        else if (k == "--showstep") r.showstep = atol(val().c_str());
        else if (k == "--savestep") r.savestep = atol(val().c_str());
        else if (k == "--basept-from") r.bp_from = num();
        else if (k == "--basept-to") r.bp_to = num();
        else if (k == "--basept-step") r.bp_step = num();
        else if (k == "--basept") {
            string s = val();
            size_t at = 0;
            while (at <= s.size()) {
                size_t c = s.find(',', at);
                if (c == string::npos) c = s.size();
                if (c > at) r.bp_list.push_back(atof(s.substr(at, c - at).c_str()));
                at = c + 1;
            }
        } else if (k == "--reinit") r.reinit = true;
        else if (k == "--out-dir") r.out_dir = val();
        else if (k == "--ca-header") r.ca_header = true;
        else if (k == "--dry-run") r.dry = true;
        else usage(("unknown option " + k).c_str());
    }
    if (r.showstep < 1 || r.savestep < 1 || r.allstep < 0) usage("step counts must be positive");
    if (!r.cocurve.empty()) r.p.cocurve_dir = r.cocurve.c_str();
    return r;
}

// The sweep values, accumulated in double exactly as the reference's loop
// (FluidCuda.cu:1264) accumulates them.
vector<double> sweep(const Run &r)
{
    if (!r.bp_list.empty()) return r.bp_list;
    vector<double> v;
    if (!(r.bp_step > 0)) return v;
    for (double b = r.bp_from; b <= r.bp_to; b += r.bp_step) v.push_back(b);
    return v;
}

string ca_file_name(const Run &r)
{
    char buf[512];
    snprintf(buf, sizeof buf, "%s/CP%s_MRT_Tau=%2.1f_FIELD%dx%dx%d_ContactAngle_R%3.1f_Tr%3.1f.txt",
             r.out_dir.c_str(), model_name(r.p.model) + 3, r.p.tau, r.p.dx, r.p.dy, r.p.dz, r.radius, r.p.tr);
    return buf;
}

long long now_ms()
{
    using namespace std::chrono;
    return duration_cast<milliseconds>(steady_clock::now().time_since_epoch()).count();
}

// Host-side state of the reference's globals that ShowData and
// SaveContactAngle print.
struct Shown {
    long step = 0;
    double mass = 0, max_speed = 0;
    double ca_left = 0, ca_right = 0, ca_cap = 0, x_left = 0, x_right = 0;
    double d0 = 0, d1 = 0, d2 = 0;  // Dens at (DX/2, 0, 3), (DX/2, DY/2/8, 3), (DX/2, DY/2/4, 3)
    long long last_ms = 0;
};

// ShowData (FluidCuda.cu:1658-1732), CONTACTANGLE build.
void show_data(const Run &r, double den_g, double den_l, double base_pt, Shown &s)
{
    if (s.step == 0) {
        cout << "程序参数设置：" << endl;
        cout << "Multiphase: " << model_name(r.p.model) << "    DX=" << r.p.dx << "    DY=" << r.p.dy
             << "    DZ=" << r.p.dz << "    Tau=" << r.p.tau << "    Tr=" << r.p.tr << "    DenG=" << den_g
             << "    DenL=" << den_l << endl;
        cout << "Radius=" << r.radius << "    Width=" << r.width << "    Ka=" << r.p.ka << "    K=" << r.p.k
             << "    BasePt=" << base_pt << "  \tAllStep=" << r.allstep << endl;
        if (r.p.complex_bc)
            cout << "化学势边界条件：逐层计算" << endl;
        else
            cout << "化学势边界条件：多层设置为相同" << endl;
        cout << "ChemicalPotential Calculation Method: ";
        cout << (r.p.lap_order == 7 ? "SevenPoint" : "FivePoint") << endl;
        cout << endl;
        cout << "NowStep" << "    Mass" << "    Den(DX/2 , 0 , 3)" << "    Den(DX/2, DY/2/8, 3)"
             << "    Den(DX/2, DY/2/4, 3)" << "    MaxSpeed" << "    CaLeft" << "    CaRight" << "    CaCap"
             << "    XLeft" << "    XRight" << "    StepTime" << endl;
        cout << "----------------------------------------------------------------------------------------------------"
             << endl;
    }
    const long long t = now_ms();
    const long long step_time = t - s.last_ms;
    s.last_ms = t;
    cout << setw(9) << s.step << "    " << setiosflags(ios::fixed) << setprecision(12) << s.mass << "    "
         << setprecision(16) << s.d0 << "    " << s.d1 << "    " << s.d2 << "    " << setprecision(6)
         << s.max_speed << "    " << s.ca_left << "    " << s.ca_right << "    " << s.ca_cap << "    " << s.x_left
         << "    " << s.x_right << "    " << step_time << endl;
}

// SaveContactAngle (FluidCuda.cu:1735-1771).
void save_contact_angle(const Run &r, double base_pt, const Shown &s, bool header)
{
    const string name = ca_file_name(r);
    ofstream f;
    if (header) {
        f.open(name, ios::app);
        f << "Droprad" << "  " << "BasePt" << "  " << "NowStep" << "  " << "CaLeft" << "  " << "CaRight" << "  "
          << "CaCap" << "  " << "XLeft" << "  " << "XRight" << "  " << endl;
        f.close();
    }
    f.open(name, ios::app);
    f << r.radius << "  " << base_pt << "  " << s.step << "  " << s.ca_left << "  " << s.ca_right << "  " << s.ca_cap
      << "  " << s.x_left << "  " << s.x_right << "  " << endl;
    f.close();
}

int check(cpmp_status st, const char *what)
{
    if (st == CPMP_OK) return 0;
    cerr << "cpmp_run: " << what << ": " << cpmp_last_error() << endl;
    return 1;
}

}  // namespace

int main(int argc, char **argv)
{
    Run r = parse(argc, argv);
    const vector<double> bps = sweep(r);
    double den_g, den_l, A, B, Tc, Rc;  // lattice-unit coexistence densities
    if (check(cpmp_coexistence(r.p.model, r.p.tr, r.p.eos_a, r.p.eos_b, r.p.eos_omega, r.p.cocurve_dir, &den_g,
                               &den_l, &A, &B, &Tc, &Rc),
              "coexistence"))
        return 1;
    if (r.dry) {
        cout << setprecision(17);
        cout << "model " << model_name(r.p.model) << " grid " << r.p.dx << " " << r.p.dy << " " << r.p.dz
             << " den_g " << den_g << " den_l " << den_l << endl;
        cout << "basept";
        for (double b : bps) cout << " " << b;
        cout << endl << "contact_angle_file " << ca_file_name(r) << endl;
        return 0;
    }
    mkdir(r.out_dir.c_str(), 0755);
    cpmp_handle *h = nullptr;
    r.p.base_pt = bps.empty() ? r.p.base_pt : bps[0];
    if (check(cpmp_create(&r.p, &h), "create")) return 1;
    double dg, dl, a_, b_, t_, rc;
    if (check(cpmp_get_eos(h, &dg, &dl, &a_, &b_, &t_, &rc), "eos")) return 1;
    cpmp_droplet d{};
    d.radius = r.radius;
    d.width = r.width;
    if (r.has_centre) {
        d.cx = r.cx;
        d.cy = r.cy;
        d.cz = r.cz;
    } else {
        d.ref_centre = 1;
    }
    if (check(cpmp_init_droplet(h, &d), "init")) return 1;
    int dims[3];
    cpmp_get_dims(h, dims);
    const size_t N = (size_t)dims[0] * dims[1] * dims[2];
    vector<double> rho(N);
    vector<unsigned char> type(N);
    if (check(cpmp_get_field(h, CPMP_FIELD_TYPE, CPMP_F64, type.data(), N), "type")) return 1;
    const int DX = dims[0], DY = dims[1], DZ = dims[2];
    auto I = [&](int i, int j, int k) { return ((size_t)i * DY + j) * DZ + k; };
    Shown s;
    s.last_ms = now_ms();
    bool err_den = false;
    double base_pt_now = 0;
    // CalcMacroCPU (FluidCuda.cu:1626-1657): mass, max |MV|, the density
    // probes ShowData prints, and the error-density report
    auto calc_macro = [&](bool with_ca) -> int {
        cpmp_diag g;
        cpmp_status st = cpmp_reduce(h, &g);
        if (st != CPMP_OK && st != CPMP_ERR_NONFINITE) return check(st, "reduce");
        if (check(cpmp_get_field(h, CPMP_FIELD_RHO, CPMP_F64, rho.data(), N * 8), "rho")) return 1;
        s.mass = g.mass;
        s.max_speed = g.max_speed;
        if (with_ca) {
            // ContactAngle(0, DY/2) (FluidCuda.cu:557-734): when the solid
            // row has no interface crossing the reference sets the angles to
            // 0 and the contact points to DY/2 but leaves CaCap as it was
            const bool found = !(g.ca_left == 0.0 && g.ca_right == 0.0);
            s.ca_left = g.ca_left;
            s.ca_right = g.ca_right;
            if (found) s.ca_cap = g.ca_cap;
            s.x_left = g.x_left;
            s.x_right = g.x_right;
            // and it writes the x-z density slice j = DY/2 it measured on
            char xz[64];
            snprintf(xz, sizeof xz, "/XZ_%f.txt", base_pt_now);
            ofstream f(r.out_dir + xz);
            f << "i   j   Den" << endl;
            for (int k = 0; k < DZ; ++k)
                for (int i = 0; i < DX; ++i) f << i << ' ' << k << ' ' << rho[I(i, DY / 2, k)] << endl;
        }
        s.d0 = rho[I(DX / 2, 0, 3 < DZ ? 3 : 0)] / rc;
        s.d1 = rho[I(DX / 2, DY / 2 / 8, 3 < DZ ? 3 : 0)] / rc;
        s.d2 = rho[I(DX / 2, DY / 2 / 4, 3 < DZ ? 3 : 0)] / rc;
        if (g.nonfinite) {
            err_den = true;
            ofstream ef(r.out_dir + "/error_Density.txt", ios::app);
            for (int i = 0; i < DX; ++i)
                for (int j = 0; j < DY; ++j)
                    for (int k = 0; k < DZ; ++k) {
                        const double v = rho[I(i, j, k)];
                        if (type[I(i, j, k)] == 1 && (v != v || v < 0))
                            ef << "Density: " << s.step << " " << i << " " << j << " " << k << " Den = " << v << endl;
                    }
        }
        if (err_den) {
            cout << " Error Density! " << endl;
            s.step = r.allstep;
        }
        return 0;
    };
    bool first = true;
    for (size_t n = 0; n < bps.size(); ++n) {
        const double bp = bps[n];
        base_pt_now = bp;
        cout << "Now the BasePt = " << bp << endl;
        if (check(cpmp_set_base_pt(h, bp), "set_base_pt")) return 1;
        if (r.reinit && !first && check(cpmp_init_droplet(h, &d), "init")) return 1;
        first = false;
        s.step = 0;
        if (calc_macro(false)) return 1;
        show_data(r, dg, dl, bp, s);
        for (s.step = 1; s.step <= r.allstep; ++s.step) {
            // run straight to the next step that shows, saves or ends
            long next = s.step;
            while (next < r.allstep && !(next % r.showstep == 0 && next % r.savestep == 0)) ++next;
            if (check(cpmp_step(h, (int)(next - s.step + 1)), "step")) return 1;
            s.step = next;
            if (s.step % r.showstep == 0 && s.step % r.savestep == 0) {
                if (calc_macro(true)) return 1;
                show_data(r, dg, dl, bp, s);
            }
            if (s.step == r.allstep) save_contact_angle(r, bp, s, r.ca_header && n == 0);
        }
    }
    cpmp_destroy(h);
    return 0;
}
