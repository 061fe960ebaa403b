#!/usr/bin/env python3
"""Generate ``csrc/libconv_filters.h``: every FP64 filter table the library and
its oracle use, derived from the decimal coefficient tables of BigDFT's
Daubechies-16 (SYM8) family.

Decimal tables (data that must be identical to the reference's):
  * SYM8_LP, SYM8_D1, SYM8_D2, SYM8_MF  -- BigDFT/WaveletFilters.rb:25-121
  * MagicFilter ``fil`` DATA literals    -- BigDFT/magicfilter_refs.f90:17-33, 61-77
  * kinetic_per_ref second-derivative     -- BigDFT/Kinetic2.rb:1000-1014
  * 3D kinetic test filter ``kin``        -- BigDFT/Kinetic_test2.rb:3-31
  * synthesis/analysis ch/cg literals     -- BigDFT/old/Synthesis.rb:32-47,
                                             BigDFT/old/AnaRotPer-2.rb:31-46

Derived tables (restated algorithms, computed here):
  * the quadrature-mirror high-pass of a low-pass filter
    (GenericConvolution2.rb:311-328): hp = reverse(lp[i] * (-1)^i);
  * polyphase even/odd splits of the low/high pairs
    (GenericConvolution2.rb:386-410, 418-436);
  * the MagicFilter-combined wavelet filters used by s1tor/rtos1
    (GenericConvolution2.rb:336-384): exact decimal convolution of the
    low/high pass with the MagicFilter, each coefficient truncated (towards
    zero) to 30 decimal places, as the reference does with
    BigDecimal#truncate(30).

  * the Poisson finite-difference first derivatives of order nord in
    {2, 4, 6, 8, 16} (BigDFT/Poisson.rb:20-166, the table c1D(-m:m,-m:m),
    m = nord/2): c1D(:, j) are the weights on the nord+1 unit-spaced nodes
    0..nord for the derivative at node m + j, i.e. Fornberg's algorithm
    (Math. Comp. 51 (1988) 699-706) in exact rational arithmetic, each
    weight rounded once to the nearest double (the reference writes each as
    one quotient of two exact doubles, which rounds the same way).  One entry
    of the reference table differs from those weights: its nord = 8 stencil
    for the first node, c1D(0,-4), is +35/2 where the weight is -35/2; it is
    kept as the reference has it, so results match the reference's.

Every decimal string is converted to the nearest double (Python ``float`` is
correctly rounded, as a C compiler's literal parsing is) and emitted with
``repr`` so the C literal round-trips to that exact double.

Usage: python gen_filters.py [output_header]
"""
from decimal import Decimal, getcontext, ROUND_DOWN
from fractions import Fraction
import os
import sys

getcontext().prec = 400  # far above what exact products of 64-digit inputs need

SYM8_LP = """
-0.003382415951005002595457699235919135128243170037709254473102252636e0
-0.000542132331800010689347836944017347858824603460398208422132403418e0
0.03169508781152599143142570752391597485717789804058994936458784274e0
0.00760748732497660819192100801219238392349477628276637389848185158e0
-0.1432942383512726628440955443992739699342280444601654901737376736e0
-0.0612733590678110778430467690736584126556319554926068967930152121e0
0.481359651259053391589568580264984525838564867578278365157821169e0
0.777185751699628028624333566639210809121328610967576793053795894e0
0.3644418948361789367595594323842960136510635625353935885398873954e0
-0.0519458381078818007357107290625634285296352747007956649813654351e0
-0.02721902991710348632196412421624687935352227243191326268168750639e0
0.0491371796737302867869109881551654429015527772546123162293717851e0
0.003808752013894489463071922223049694342708315178928653470691661633e0
-0.01495225833706219911849029822472598879079395753054027354116270039e0
-0.0003029205147241330812639124399571849886852187149285126161207667492e0
0.001889950332767689184274432603245581173345564367859597144366089742e0
""".split()

SYM8_D1 = """
1.585464751677102510097179308121926878193105545088903963493188933e-19
-1.240078536096648534547438612731567439237828505396469976633162949e-14
7.252206916665149851135591529994603533072998149301256702737646004e-13
9.697184925637300947553068758362746388131353737840306778881714191e-10
7.207948238588481597101904067961163265788433149563519306241683057e-8
-3.993810456408053712133667496514167576517175934074503260991290434e-8
-2.451992111053665419191564123434446284949933594307826864375530275e-7
-0.00007667706908380351933901775234801819926013328778633133146782374641e0
0.001031530213375445369097964780217146384828800932615832761481602166e0
-0.006958379116450707495020407536758241511060163284033091893516844663e0
0.03129014783948023634381563995259325360348542944538434049761056972e0
-0.1063640682894442760934532284702982844094052663346279226663978027e0
0.3032593514765938346887962440931660566677778365072429185627922116e0
-0.8834460460908270942785855643941098713157598590915435134511547387e0
0e0
0.8834460460908270942785855643941098713157598590915435134511547387e0
-0.3032593514765938346887962440931660566677778365072429185627922116e0
0.1063640682894442760934532284702982844094052663346279226663978027e0
-0.03129014783948023634381563995259325360348542944538434049761056972e0
0.006958379116450707495020407536758241511060163284033091893516844663e0
-0.001031530213375445369097964780217146384828800932615832761481602166e0
0.00007667706908380351933901775234801819926013328778633133146782374641e0
2.451992111053665419191564123434446284949933594307826864375530275e-7
3.993810456408053712133667496514167576517175934074503260991290434e-8
-7.207948238588481597101904067961163265788433149563519306241683057e-8
-9.697184925637300947553068758362746388131353737840306778881714191e-10
-7.252206916665149851135591529994603533072998149301256702737646004e-13
1.240078536096648534547438612731567439237828505396469976633162949e-14
-1.585464751677102510097179308121926878193105545088903963493188933e-19
""".split()

SYM8_D2 = """
-6.924474940639200152025730585882115968579663856946045039077208122e-18
2.708004936263194382698566890376475760883688432060067551662628469e-13
-5.813879830282540547959250667464887365484326600877085719823602219e-11
-1.058570554967414703734941322870242653300359680996853899470022889e-8
-3.723076304736927584879149697304408803274215476409064356088861068e-7
2.09042349529203659579228894473609842180443353287738050051136428e-6
-0.00002398228524507599670405555359023134858523138758236007644059252025e0
0.000451679202875022353494800376397584960775566033384647821996975667e0
-0.004097656893426338238993270511883154847227992660459896521032712738e0
0.02207029188482255523789911295638968408882184950053649882554342682e0
-0.0822663999742123340987663520631668159519522793487327848931628121e0
0.2371780582153805636239247475762231531845465033753480080361580487e0
-0.6156141465570069496314853948700762181701834843585057391570819072e0
2.219146593891116389879454640457705235616912723375223389717990369e0
-3.553692289913190194129680937424076424953761573153458649028535991e0
2.219146593891116389879454640457705235616912723375223389717990369e0
-0.6156141465570069496314853948700762181701834843585057391570819072e0
0.2371780582153805636239247475762231531845465033753480080361580487e0
-0.0822663999742123340987663520631668159519522793487327848931628121e0
0.02207029188482255523789911295638968408882184950053649882554342682e0
-0.004097656893426338238993270511883154847227992660459896521032712738e0
0.000451679202875022353494800376397584960775566033384647821996975667e0
-0.00002398228524507599670405555359023134858523138758236007644059252025e0
2.09042349529203659579228894473609842180443353287738050051136428e-6
-3.723076304736927584879149697304408803274215476409064356088861068e-7
-1.058570554967414703734941322870242653300359680996853899470022889e-8
-5.813879830282540547959250667464887365484326600877085719823602219e-11
2.708004936263194382698566890376475760883688432060067551662628469e-13
-6.924474940639200152025730585882115968579663856946045039077208122e-18
""".split()

SYM8_MF = """
2.727344929119796596577153130172279928753156083478007592916189e-6
-0.00005185986881173432922848639136911486874128383207856851537290756e0
0.0004944322768868991919228225947675097243713535139015057534937039e0
-0.003441281444934938572808815096868218611693146749743898558729002e0
0.013372634148547947527334234670132209969450042970835150850985441e0
-0.02103025160930381434955489412839065067238766803542905035107527e0
-0.06048952891969835160028346363993374032323310579329060307398682e0
0.99404156978340039931786167125707312696826875197808439082533262e0
0.06126258958312079821953805969111734845421975622016765542503018e0
0.02373821463724942397566389712597274534984899296281082155336152e0
-0.00942047030201080385922711540948195074607340327611386232053071e0
0.001747237136729939034494478127498529416920979083511241686685502e0
-0.000301580381326904631671637038261698791032841826554967601640246e0
0.000087629844762105595646891618941163970464425424613649618138794e0
-0.00001290557201342060969516786758559028264129757158423127355882943e0
8.4334247333529341094733325815816232969177478728797427310317e-7
""".split()

# magicfilter_per_ref / magicfilter_free_ref DATA fil(-8:7)
MF_FORTRAN = """
8.4334247333529341094733325815816e-7
-0.1290557201342060969516786758559028e-4
0.8762984476210559564689161894116397e-4
-0.30158038132690463167163703826169879e-3
0.174723713672993903449447812749852942e-2
-0.942047030201080385922711540948195075e-2
0.2373821463724942397566389712597274535e-1
0.612625895831207982195380597e-1
0.9940415697834003993178616713
-0.604895289196983516002834636e-1
-0.2103025160930381434955489412839065067e-1
0.1337263414854794752733423467013220997e-1
-0.344128144493493857280881509686821861e-2
0.49443227688689919192282259476750972e-3
-0.5185986881173432922848639136911487e-4
2.72734492911979659657715313017228e-6
""".split()

# kinetic_per_ref fil(0:14) before scaling (symmetric: fil(-i) = fil(i))
KIN_FORTRAN = """
-3.5536922899131901941296809374e0
2.2191465938911163898794546405e0
-0.6156141465570069496314853949e0
0.2371780582153805636239247476e0
-0.0822663999742123340987663521e0
0.02207029188482255523789911295638968409e0
-0.409765689342633823899327051188315485e-2
0.45167920287502235349480037639758496e-3
-0.2398228524507599670405555359023135e-4
2.0904234952920365957922889447361e-6
-3.7230763047369275848791496973044e-7
-1.05857055496741470373494132287e-8
-5.813879830282540547959250667e-11
2.70800493626319438269856689037647576e-13
-6.924474940639200152025730585882e-18
""".split()

# synthesis_*_ref / analysis_*_ref DATA ch(-7:8), cg(-7:8) (the zero pads of
# the synthesis ch(-8:9)/cg(-8:9) are added by the consumers)
CH_FORTRAN = """
-0.0033824159510050025955 -0.00054213233180001068935 0.031695087811525991431
0.0076074873249766081919 -0.14329423835127266284 -0.061273359067811077843
0.48135965125905339159 0.77718575169962802862 0.36444189483617893676
-0.051945838107881800736 -0.027219029917103486322 0.049137179673730286787
0.0038087520138944894631 -0.014952258337062199118 -0.00030292051472413308126
0.0018899503327676891843
""".split()
CG_FORTRAN = """
-0.0018899503327676891843 -0.00030292051472413308126 0.014952258337062199118
0.0038087520138944894631 -0.049137179673730286787 -0.027219029917103486322
0.051945838107881800736 0.36444189483617893676 -0.77718575169962802862
0.48135965125905339159 0.061273359067811077843 -0.14329423835127266284
-0.0076074873249766081919 0.031695087811525991431 0.00054213233180001068935
-0.0033824159510050025955
""".split()


def neg(s):
    """Sign flip of a decimal string, as the reference does on strings."""
    return s[1:] if s.startswith('-') else '-' + s


def qmf_high(lp):
    """High-pass partner: alternate signs then reverse (GenericConvolution2.rb:311-328)."""
    return [e if i % 2 == 0 else neg(e) for i, e in enumerate(lp)][::-1]


def combine(lp_str, mf_str, cv_center):
    """MagicFilter-combined low/high filters (GenericConvolution2.rb:336-384).

    Returns (center, low_strings, high_strings); each coefficient is the exact
    decimal sum truncated to 30 decimal places."""
    lp = [Decimal(e) for e in lp_str]
    hp = [(e if i % 2 == 0 else -e) for i, e in enumerate(lp)][::-1]
    cv = [Decimal(e) for e in mf_str]
    n_lp, n_cv = len(lp), len(cv)
    lp_c = n_lp // 2
    cv_b = (-cv_center, n_cv - cv_center - 1)
    lp_b = (-lp_c, n_lp - lp_c - 1)

    def bounds():
        lo, hi = cv_b[0] - lp_b[1], cv_b[1] - lp_b[0]
        if lo % 2 != 0:
            lo -= 1
        if hi % 2 == 0:
            hi += 1
        return lo, hi

    lo, hi = bounds()
    q = Decimal('1e-30')

    def conv(f):
        out = []
        for i in range(lo, hi + 1):
            s = Decimal(0)
            for j in range(lp_b[0], lp_b[1] + 1):
                k = i - j - 1 + cv_center
                if 0 <= k < n_cv:
                    s += f[j + lp_c] * cv[k]
            out.append(s.quantize(q, rounding=ROUND_DOWN))
        return out

    return -lo, [str(v) for v in conv(lp)], [str(v) for v in conv(hp)]


def split(low, high, reverse, center_half):
    """Polyphase split (GenericConvolution2.rb:386-410): (le, lo, he, ho, lowfil)."""
    li = low[::-1] if reverse else low
    hi = high[::-1] if reverse else high
    return li[0::2], li[1::2], hi[0::2], hi[1::2], -center_half


def wavelet_sets():
    """Polyphase filters for every (wavelet op, BC family) the library serves.

    Keys: (name, direction, family) with family 'p' (periodic / free no-grow)
    or 'gs' (grow / shrink; only the combined filters differ)."""
    sets = {}
    lp, hp = SYM8_LP, qmf_high(SYM8_LP)
    center = len(lp) // 2
    center -= center % 2
    for fam in ('p', 'gs'):
        sets[('sym8', 'dec', fam)] = split(lp, hp, False, center // 2) + (len(lp),)
        sets[('sym8', 'rec', fam)] = split(lp, hp, True, (len(lp) - center - 1) // 2) + (len(lp),)
    for fam, cvc in (('p', 8), ('gs', 7)):
        c, lo_, hi_ = combine(SYM8_LP, SYM8_MF, cvc)
        sets[('symicomb8', 'dec', fam)] = split(lo_, hi_, False, c // 2) + (len(lo_),)
        sets[('symicomb8', 'rec', fam)] = split(lo_, hi_, True, (len(lo_) - c - 1) // 2) + (len(lo_),)
    return sets


FD_ORDERS = (2, 4, 6, 8, 16)
FD_NTAPS = 17          # every central stencil padded to 17 taps (lowfil -8)


def fornberg(z, nodes):
    """Exact first-derivative weights at z on `nodes` (Fornberg 1988, m = 1)."""
    n = len(nodes) - 1
    c = [[Fraction(0), Fraction(0)] for _ in range(n + 1)]
    c[0][0] = Fraction(1)
    c1, c4 = Fraction(1), Fraction(nodes[0] - z)
    for i in range(1, n + 1):
        mn = min(i, 1)
        c2, c5, c4 = Fraction(1), c4, Fraction(nodes[i] - z)
        for j in range(i):
            c3 = Fraction(nodes[i] - nodes[j])
            c2 *= c3
            if j == i - 1:
                for k in range(mn, 0, -1):
                    c[i][k] = c1 * (k * c[i - 1][k - 1] - c5 * c[i - 1][k]) / c2
                c[i][0] = -c1 * c5 * c[i - 1][0] / c2
            for k in range(mn, 0, -1):
                c[j][k] = (c4 * c[j][k] - k * c[j][k - 1]) / c3
            c[j][0] = c4 * c[j][0] / c3
        c1 = c2
    return [c[i][1] for i in range(n + 1)]


def fd_table(nord):
    """c1D(:, j) for j = -m..m (rows), weights on nodes 0..nord (columns)."""
    m = nord // 2
    rows = [fornberg(m + j, list(range(nord + 1))) for j in range(-m, m + 1)]
    if nord == 8:
        rows[0][4] = -rows[0][4]          # the reference's c1D(0,-4) = +35/2
    return rows


def carr(name, vals):
    body = ',\n  '.join(repr(float(v)) for v in vals)
    return f"static const double {name}[{len(vals)}] = {{\n  {body}\n}};\n"


def generate():
    out = []
    out.append("/* Generated by gen_filters.py from the decimal SYM8 tables; do not edit.\n"
               " * Every value is the double nearest to the reference's decimal string. */\n"
               "#pragma once\n\n")
    out.append(carr("LCG_SYM8_LP", SYM8_LP))
    out.append(carr("LCG_SYM8_D1", SYM8_D1))
    out.append(carr("LCG_SYM8_D2", SYM8_D2))
    out.append(carr("LCG_SYM8_MF", SYM8_MF))
    out.append(carr("LCG_MF_FORTRAN", MF_FORTRAN))
    out.append(carr("LCG_KIN_FORTRAN", KIN_FORTRAN))
    out.append(carr("LCG_CH_FORTRAN", CH_FORTRAN))
    out.append(carr("LCG_CG_FORTRAN", CG_FORTRAN))
    # ConvolutionFilter tables (taps in ascending l, from lowfil):
    #   sym8_md  = reverse(SYM8_MF), centre 8  -> lowfil -8  (LibconvBase.rb:238-242)
    #   sym8_imd = SYM8_MF,          centre 7  -> lowfil -7  (LibconvBase.rb:244-248)
    #   sym8_d2  = SYM8_D2,          centre 14 -> lowfil -14 (Kinetic1d.rb:32)
    #   sym8_d1  = SYM8_D1,          centre 14 -> lowfil -14
    out.append(carr("LCG_CONV_SYM8_MD", SYM8_MF[::-1]))
    out.append(carr("LCG_CONV_SYM8_IMD", SYM8_MF))
    out.append("#define LCG_CONV_SYM8_MD_LOWFIL (-8)\n#define LCG_CONV_SYM8_IMD_LOWFIL (-7)\n"
               "#define LCG_CONV_SYM8_D2_LOWFIL (-14)\n#define LCG_CONV_SYM8_D1_LOWFIL (-14)\n\n")
    flat, offs = [], []

    def put(tag, vals):
        offs.append((tag, len(flat)))
        flat.extend(float(v) for v in vals)

    put('MD', SYM8_MF[::-1])
    put('IMD', SYM8_MF)
    put('D1', SYM8_D1)
    put('D2', SYM8_D2)
    # Poisson central stencils c1D(:,0), zero-padded to 17 taps at lowfil -8
    out.append("/* Poisson finite differences (nord 2..16): central stencils in the flat\n"
               " * table (17 taps, lowfil -8, zero padded); one-sided stencils c1D(:,j),\n"
               " * j = -m..m, row after row, in LCG_FD_EDGE at LCG_FD_EDGE_OFF_<nord>. */\n"
               f"#define LCG_FD_NTAPS ({FD_NTAPS})\n#define LCG_FD_LOWFIL (-8)\n")
    edge, edge_offs = [], []
    for nord in FD_ORDERS:
        rows = fd_table(nord)
        m = nord // 2
        central = [Fraction(0)] * (8 - m) + rows[m] + [Fraction(0)] * (8 - m)
        put(f'FD{nord}', central)
        edge_offs.append((nord, len(edge)))
        for r in rows:
            edge.extend(float(v) for v in r)
    for nord, off in edge_offs:
        out.append(f"#define LCG_FD_EDGE_OFF_{nord} {off}\n")
    out.append(f"#define LCG_FD_EDGE_N {len(edge)}\n")
    out.append("#define LCG_FD_EDGE_INIT { \\\n  " +
               ", \\\n  ".join(repr(v) for v in edge) + " }\n")
    for (name, d, fam), (le, lo, he, ho, lowfil, length) in sorted(wavelet_sets().items()):
        tag = f"LCG_WT_{name.upper()}_{d.upper()}_{fam.upper()}"
        out.append(f"/* {name} {d} ({'periodic/free' if fam == 'p' else 'grow/shrink'}): "
                   f"polyphase taps lowfil={lowfil}..upfil={lowfil + len(le) - 1}, "
                   f"full low-pass length {length} */\n")
        out.append(f"#define {tag}_LOWFIL ({lowfil})\n#define {tag}_NTAPS ({len(le)})\n"
                   f"#define {tag}_LENGTH ({length})\n")
        out.append(carr(f"{tag}_LE", le))
        out.append(carr(f"{tag}_LO", lo))
        out.append(carr(f"{tag}_HE", he))
        out.append(carr(f"{tag}_HO", ho))
        # flat order for the GPU table: LE, LO, HE, HO, each ntaps long
        put(tag[len('LCG_'):], list(le) + list(lo) + list(he) + list(ho))
    out.append("\n/* One flat table (device constant memory): offsets of each filter. */\n")
    for tag, off in offs:
        out.append(f"#define LCG_FTAB_{tag} {off}\n")
    out.append(f"#define LCG_FTAB_N {len(flat)}\n")
    out.append("#define LCG_FTAB_INIT { \\\n  " +
               ", \\\n  ".join(repr(v) for v in flat) + " }\n")
    return ''.join(out)


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    dest = sys.argv[1] if len(sys.argv) > 1 else os.path.join(here, 'csrc', 'libconv_filters.h')
    text = generate()
    old = open(dest).read() if os.path.exists(dest) else None
    if old != text:
        with open(dest, 'w') as f:
            f.write(text)


if __name__ == '__main__':
    main()
