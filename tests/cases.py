"""Problem set shared by the CPU and GPU parity tests (Olliptic.x command lines)."""
from ollipticid_gb300 import parse_olliptic_args

CASES = {
    # single boosted puncture, the reference's config-1 geometry at fewer levels
    "o2_single": "-eq Punctures -B Robin -NumBH 1 -bhmp1 0.5 -bhpx1 0.1 -L 64 -N 33 -O 2 -l 4 -nu2 20",
    "o4_spin": "-eq Punctures -B Robin -NumBH 1 -bhmp1 0.5 -bhpx1 0.1 -bhsz1 0.1 -L 40 -N 25 -O 4 -l 3 -nu2 5",
    "o6_boost_y": "-eq Punctures -B Robin -NumBH 1 -bhmp1 0.5 -bhpy1 0.1 -bhsx1 0.05 -L 40 -N 25 -O 6 -l 3 -nu2 5",
    "o8_offset": "-eq Punctures -B Robin -NumBH 1 -bhmp1 0.5 -bhpz1 0.1 -bhx1 0.3 -L 40 -N 25 -O 8 -l 3 -nu2 5",
    # equal-mass binary whose coarse refinement boxes merge (off-lattice centres)
    "o4_binary_merge": ("-eq Punctures -B Robin -NumBH 2 -bhmp1 0.487209 -bhy1 3 -bhpx1 -0.09 -bhmp2 0.487209 "
                        "-bhy2 -3 -bhpx2 0.09 -L 40 -N 25 -O 4 -l 4 -nu2 5"),
    # puncture + scalar field (ps_case 2 has the potential term e != 0)
    "sf_binary": ("-eq Punctures_scalar_field -B Robin -NumBH 2 -bhmp1 0.487209 -bhy1 3 -bhpx1 -0.09 "
                  "-bhmp2 0.487209 -bhy2 -3 -bhpx2 0.09 -L 40 -N 25 -O 2 -l 4 -nu2 5 -psc 2 -phi0 0.02 -r0 8 -sigma 4"),
}

CONFIG1 = "-eq Punctures -B Robin -NumBH 1 -bhmp1 0.5 -bhpx1 0.1 -L 64 -N 33 -O 2 -l 6 -s 1e-10 -nu2 20"
CONFIG2 = ("-eq Punctures -B Robin -BA 0.0 -Bn 1 -NumBH 2 -bhmp1 0.487209 -bhy1 5.5 -bhpx1 -0.0901099 "
           "-bhpy1 -0.000703975 -bhmp2 0.487209 -bhy2 -5.5 -bhpx2 0.0901099 -bhpy2 0.000703975 "
           "-L 1000 -N 65 -O 4 -l 9 -s 1e-11 -Dp 0.05 -nu2 20")
CONFIG3 = CONFIG2.replace("-N 65", "-N 129").replace("-O 4", "-O 8").replace("-s 1e-11", "-s 1e-10")


def problem(name_or_args: str):
    args = CASES.get(name_or_args, name_or_args)
    return parse_olliptic_args(args.split())
