"""Runs an AMDAT command script through the C oracle and renders the output
files the reference writes (test-side checker).

Formats follow the reference writers: Mean_Square_Displacement::write
(mean_square_displacement.cpp:186), Non_Gaussian_Parameter::write,
Correlation_2D::write (correlation_2d.cpp:475-504),
Space_Time_Correlation_Function::write (space_time_correlation_function.cpp:240),
Structure_Factor::write (structure_factor.cpp:323-344),
Radial_Distribution_Function::write (radial_distribution_function.cpp:326),
Mean_Square_Displacement_2D::write (mean_square_displacement_2d.cpp:183),
Mean_Displacement::write (mean_displacement.cpp:185), DebyeWaller_Dist::write
(debyewaller_dist.cpp:101) and Displacement_Distribution::write
(displacement_distribution.cpp:103).
"""
from __future__ import annotations

import numpy as np

from amdat_files import fmt
from oracle import oracle as orc
from oracle import wavevectors as wv

VERSION = "1.0.1"
f32 = np.float32


class OracleRun:
    def __init__(self, traj, qvec, mode=orc.REF32):
        self.traj = traj
        self.mode = mode
        self.qn, self.qoff = qvec
        self.unwrapped = np.ascontiguousarray(traj.unwrapped, np.float32)
        self.wrapped = traj.wrapped()
        self.limit = 0
        self.lists = {}
        self.files = {}
        self.flags = {}
        self.stored = {}
        self.bins = {}
        self.last_vhs = None
        self.gc = None

    def scheme(self):
        return orc.scheme(self.traj.scheme, self.limit)

    def shells(self, m0, m1):
        kv = self.qn[self.qoff[m0]:self.qoff[m1 + 1]]
        off = self.qoff[m0:m1 + 2] - self.qoff[m0]
        return kv, off

    def min_box(self):
        return float(f32(self.traj.box.min()))

    def run(self, script: str):
        lines = [ln.strip() for ln in script.splitlines() if ln.strip()]
        i = 0
        while i < len(lines):
            toks = lines[i].split()
            i += 1
            # '\\x...' tokens are flags (Tokenize::parse_token with the '\\' marker)
            self.flags = {t[1]: t[2:] for t in toks if len(t) >= 2 and t[0] == "\\"}
            a = [t for t in toks if not (len(t) >= 2 and t[0] == "\\")]
            cmd = a[0]
            if cmd == "structure_factor_from_rdf":
                self.cmd_structure_factor_from_rdf(a)
                continue
            if cmd == "create_list":
                sel = lines[i].split()
                i += 1
                self.lists[a[1]] = self.select(sel)
                continue
            if cmd == "limit":
                self.limit = int(a[1])
                continue
            if cmd == "create_bin_list":
                self.bins[a[1]] = self.make_bins(lines[i].split())
                i += 1
                continue
            target = lines[i].split()
            i += 1
            if target[0] == "bin_list":
                self.run_bins(cmd, a, target)
                continue
            lst = self.lists[target[1]]
            if isinstance(lst, dict):  # time-dependent list (find_fast)
                self.run_timelist(cmd, a, lst)
                continue
            getattr(self, "cmd_" + cmd)(a, lst)
        return self.files

    # --- compare_gaussian / find_fast (src/control.cpp:3378-3500) ---
    def cmd_compare_gaussian(self, a, lst):
        """Gaussian_Comparison (gaussian_comparison.cpp), float storage and double pow/exp."""
        import math
        s = self.scheme()
        msd = orc.msd(s, self.unwrapped, lst, self.mode)
        ngp = orc.ngp(s, self.unwrapped, lst, self.mode)
        if len(a) == 3:
            ti = int(a[2])
        else:
            ti, best = -1, f32(0)
            for g in range(1, len(ngp)):
                if f32(ngp[g]) > best:
                    best, ti = f32(ngp[g]), g
        v = self.last_vhs
        nb, bs = v["nb"], v["bs"]
        PI = 3.14159265
        alpha = f32(3.0 / (2.0 * float(f32(msd[ti]))))
        gauss, vh = [], []
        for b in range(nb):
            shell = f32(4.0 / 3.0 * PI * (math.pow((float(f32(b)) + 1.0) * float(bs), 3.0)
                                          - math.pow(float(f32(f32(b) * bs)), 3.0)))
            vh.append(f32(f32(v["corr"][ti][b]) * shell))
            r = (float(f32(b)) + .5) * float(bs)
            gauss.append(f32(math.pow(float(alpha) / PI, 1.5) * math.exp(-float(alpha) * math.pow(r, 2.0))
                             * float(shell)))
        si = fi = 0
        for b in range(1, nb):
            if gauss[b] >= vh[b]:
                si = b - 1
                break
        for b in range(si + 1, nb):
            if gauss[b] <= vh[b]:
                fi = b
                break
        slowb = f32(math.pow((float(f32(si)) + .5) * float(bs), 2.0))
        fastb = f32(math.pow((float(f32(fi)) - .5) * float(bs), 2.0))
        slow = gslow = f32(0)
        for b in range(1, si + 1):
            slow = f32(slow + vh[b])
            gslow = f32(gslow + gauss[b])
        fast, gfast = f32(1.0 - float(slow)), f32(1.0 - float(gslow))
        for b in range(si + 1, fi):
            fast = f32(fast - vh[b])
            gfast = f32(gfast - gauss[b])
        self.gc = dict(ti=ti, fastb=fastb)
        t = self.times(s)
        txt = ""
        if fi == 0:
            txt += ("Warning: program cannot identify two crossing points between self Van Hove and Gaussian "
                    "approximation self Van Hove.  Fractions of slow and fast particles will be incorrect.\n")
        txt += f"Gaussian comparison data created by AMDAT v.{VERSION}\n"
        txt += f"t*\n{fmt(t[ti])}\n"
        txt += f"Slow_Cutoff: {fmt(math.pow(float(slowb), 0.5))}\nFast_Cutoff: {fmt(math.pow(float(fastb), 0.5))}\n"
        txt += "\tSlow_Fraction\tFast_Fraction\n"
        txt += f"Gaussian\t{fmt(gslow)}\t{fmt(gfast)}\nActual\t{fmt(slow)}\t{fmt(fast)}\n"
        txt += f"Excess\t{fmt(f32(slow - gslow))}\t{fmt(f32(fast - gfast))}\n\n"
        txt += "Self_Van_Hove*shellvolume\nradius\tgaussian\tactual\n"
        for b in range(nb):
            txt += f"{fmt((b + .5) * float(bs))}\t{fmt(gauss[b])}\t{fmt(vh[b])}\n"
        self.files[self.name(a[1])] = txt

    def _fast(self, a, lst, gap, threshold):
        s = self.scheme()
        fast, bins = orc.fast_particles(s, self.unwrapped, lst, gap, float(threshold))
        counts = fast.sum(axis=1)
        nb = len(counts)
        avg = 0.0
        for c in counts:
            avg += float(c) / float(nb)
        times = self.traj.scheme.timelist()
        K, frt = self.traj.scheme.n_exponential_steps, self.traj.scheme.frt
        txt = f"Average_trajectories:\t{fmt(avg)}\nCount_List\n"
        txt += "".join(f"{fmt(times[b * K + frt])}\t{int(c)}\n" for b, c in enumerate(counts))
        self.files[self.name(a[2])] = txt
        self.lists[a[1]] = dict(bins=bins)

    def cmd_find_fast(self, a, lst):
        self._fast(a, lst, self.gc["ti"], self.gc["fastb"])

    def cmd_find_fast_fixedthreshold(self, a, lst):
        self._fast(a, lst, int(a[3]), f32(float(a[4])))

    def run_timelist(self, cmd, a, td):
        """msd / ngp / isfs over a time-dependent list: members at each start frame."""
        s = self.scheme()
        allat = np.arange(self.traj.n_atoms, dtype=np.int32)
        if cmd == "msd":
            m, _ = orc.msd_bins(s, self.unwrapped, allat, td["bins"], 1, 0, self.mode)
            self.files[self.name(a[1])] = self.msd_text(m[0], s)
        elif cmd == "ngp":
            q = orc.ngp_bins(s, self.unwrapped, allat, td["bins"], 1, 0, self.mode)[0]
            t = self.times(s)
            txt = f"Non-Gaussian parameter data created by AMDAT v.{VERSION}\n"
            self.files[self.name(a[1])] = txt + "".join(f"{fmt(t[g])}\t{fmt(f32(q[g]))}\n" for g in range(len(t)))
        elif cmd == "isfs":
            m0, m1 = int(a[2]), int(a[3])
            maxlen = float(a[5])
            fb = int(a[6]) if len(a) > 6 else 0
            L = maxlen if maxlen > 0 else self.min_box()
            sp = wv.spacing(L)
            kv, off = self.shells(m0, m1)
            corr = orc.isfs_bins(s, self.unwrapped, allat, kv, off, float(sp), L, td["bins"], 1, fb, 0, self.mode)
            self.files[self.name(a[1])] = self.correlation_2d(sp, m0, m1, corr[0], s)
        elif cmd == "msd_2d":
            plane = {"xy": 0, "xz": 1, "yz": 2}[a[2]]
            m = orc.msd2d_bins(s, self.unwrapped, allat, plane, td["bins"], 1, 0, self.mode)
            self.files[self.name(a[1])] = self.msd2d_text(a[2], m[0], s)
        elif cmd == "mean_displacement":
            md = orc.mean_disp_bins(s, self.unwrapped, allat, td["bins"], 1, 0, self.mode)
            self.files[self.name(a[1])] = self.md_text(md[0], s)
        else:
            raise ValueError(cmd)

    # --- spatial bins (Control::create_bin_list, src/control.cpp:3841-4000) ---
    def box_bounds(self):
        lo = self.traj.box_lo.astype(np.float32)
        hi = (self.traj.box_lo.astype(np.float64) + self.traj.box.astype(np.float64)).astype(np.float32)
        return lo, hi

    def make_bins(self, spec):
        lo, hi = self.box_bounds()
        if spec[0] == "distance":
            self.wrapped = orc.boxify(self.wrapped, lo, hi)  # System::boxify, kept for later commands
            return self.distance_bins(spec, lo, hi)
        n = [int(spec[1]), int(spec[2]), int(spec[3])]
        if spec[0] == "all":
            rlo, rhi = lo.copy(), hi.copy()
        elif spec[0] == "region":
            # Trajectory_List_Bins region constructor (src/trajectory_list_bins.cpp:308-357):
            # a bound of 0, or one outside the box, is the box's own
            v = [f32(float(x)) for x in spec[4:10]]
            rlo = np.array([lo[d] if (v[2 * d] == 0 or v[2 * d] < lo[d]) else v[2 * d] for d in range(3)], np.float32)
            rhi = np.array([hi[d] if (v[2 * d + 1] == 0 or v[2 * d + 1] > hi[d]) else v[2 * d + 1] for d in range(3)],
                           np.float32)
        else:
            raise ValueError(spec)
        self.wrapped = orc.boxify(self.wrapped, lo, hi)  # System::boxify, kept for later commands
        return dict(n=n, bins=orc.assign_bins(self.wrapped, n, rlo, rhi))

    def distance_bins(self, spec, lo, hi):
        """create_bin_list distance trajectory|point|plane (src/control.cpp:3915-3990)
        with the bin-count limits of the Trajectory_List_Bins constructors
        (src/trajectory_list_bins.cpp:461-560, 560-765, 766-948)."""
        box = (hi - lo).astype(np.float32)  # boundaries: hi - lo per axis
        half = (box / f32(2)).astype(np.float32)

        def diag_limit(th):
            # pow(pow(x,2) + pow(y,2) + pow(z,2), .5) in double, stored to float
            d = f32(float(np.sqrt(sum(float(h) ** 2 for h in half))))
            return int(f32(d / th)) + 1

        sub = spec[1]
        if sub == "trajectory":  # distance trajectory <list> <from list> <thickness> <n_bins>
            th, nb = f32(float(spec[4])), int(spec[5])
            nz = min(nb, diag_limit(th))
            bins = orc.bins_distance(self.wrapped, box, 0, self.lists[spec[2]], self.lists[spec[3]],
                                     thickness=th, n_bins=nz)
            return dict(n=[1, 1, nz], bins=bins)
        if sub == "point":  # distance point <list> <x> <y> <z> <thickness> <n_bins>
            th, nb = f32(float(spec[6])), int(spec[7])
            nz = min(nb, diag_limit(th))
            pt = np.array([float(v) for v in spec[3:6]], np.float32)
            bins = orc.bins_distance(self.wrapped, box, 1, self.lists[spec[2]], point=pt, thickness=th,
                                     n_bins=nz)
            return dict(n=[1, 1, nz], bins=bins)
        if sub == "plane":  # distance plane <direction> <list> <axis> <position> <thickness> <n_bins>
            direction = {"average": 0, "above": 1, "below": 2}[spec[2]]
            axis = {"x": 0, "y": 1, "z": 2}[spec[4]]
            pos, th, nb = f32(float(spec[5])), f32(float(spec[6])), int(spec[7])
            extent = half[axis] if direction == 0 else box[axis]
            nb = min(nb, int(f32(extent / th)) + 1)
            bins = orc.bins_distance(self.wrapped, box, 2, self.lists[spec[3]], axis=axis, direction=direction,
                                     position=pos, thickness=th, n_bins=nb)
            n = [1, 1, 1]
            n[axis] = nb
            return dict(n=n, bins=bins)
        raise ValueError(spec)

    @staticmethod
    def bin_names(stem, n, sep):
        """Bin_Static_Analysis::write / Bin_Dynamics_Analysis::write file names.  Each
        index is written with `ss << i; ss.seekp(0)` into one stringstream per axis,
        so a shorter number overwrites only the front of a longer one."""
        def put(buf, v):
            t = str(v)
            return t if len(t) >= len(buf) else t + buf[len(t):]
        out = []
        sx = sy = sz = ""
        for x in range(n[0]):
            for y in range(n[1]):
                for z in range(n[2]):
                    sx, sy, sz = put(sx, x), put(sy, y), put(sz, z)
                    out.append(((x * n[1] + y) * n[2] + z, f"{stem}_bin_{sx}{sep}{sy}{sep}{sz}.bindata"))
        return out

    def run_bins(self, cmd, a, target):
        spec = self.bins[target[1]]
        lst = self.lists[target[2]]
        persist = len(target) >= 4 and int(target[3]) != 0  # msd and isfs are dynamic analyses
        n = spec["n"]
        B = n[0] * n[1] * n[2]
        s = self.scheme()
        if cmd == "msd":
            m, _ = orc.msd_bins(s, self.unwrapped, lst, spec["bins"], B, int(persist), self.mode)
            texts = [self.msd_text(m[b], s) for b in range(B)]
        elif cmd == "isfs":
            m0, m1 = int(a[2]), int(a[3])
            maxlen = float(a[5])
            fb = int(a[6]) if len(a) > 6 else 0
            L = maxlen if maxlen > 0 else self.min_box()
            sp = wv.spacing(L)
            kv, off = self.shells(m0, m1)
            corr = orc.isfs_bins(s, self.unwrapped, lst, kv, off, float(sp), L, spec["bins"], B, fb,
                                 int(persist), self.mode)
            texts = [self.correlation_2d(sp, m0, m1, corr[b], s) for b in range(B)]
        elif cmd == "msd_2d":
            plane = {"xy": 0, "xz": 1, "yz": 2}[a[2]]
            m = orc.msd2d_bins(s, self.unwrapped, lst, plane, spec["bins"], B, int(persist), self.mode)
            texts = [self.msd2d_text(a[2], m[b], s) for b in range(B)]
        elif cmd == "mean_displacement":
            md = orc.mean_disp_bins(s, self.unwrapped, lst, spec["bins"], B, int(persist), self.mode)
            texts = [self.md_text(md[b], s) for b in range(B)]
        elif cmd == "structure_factor":
            # a static analysis: Bin_Static_Analysis whatever the target line's persistence
            persist = False
            kv, off, sp, L, ts = self.sk_shells(a)
            S = orc.structure_factor_bins(s, ts, self.wrapped, lst, spec["bins"], B, kv, off, float(sp), L,
                                          self.mode)
            texts = [self.sk_text(S[b], kv, off, sp) for b in range(B)]
        else:
            raise ValueError(cmd)
        for b, name in self.bin_names(self.name(a[1]), n, "." if persist else "_"):
            self.files[name] = texts[b]

    def msd2d_text(self, plane, m, s):
        t = self.times(s)
        txt = f"2-D mean square displacement data for {plane} plane created by AMDAT v.{VERSION}\n"
        return txt + "".join(f"{fmt(t[g])}\t{fmt(f32(m[g]))}\n" for g in range(len(t)))

    def md_text(self, md, s):
        t = self.times(s)
        txt = f"Mean displacement data created by AMDAT v.{VERSION}\n"
        return txt + "".join(f"{fmt(t[g])}\t" + "\t".join(fmt(f32(v)) for v in md[g]) + "\n"
                             for g in range(len(t)))

    def msd_text(self, m, s):
        t = self.times(s)
        txt = f"Mean square displacement data created by AMDAT v.{VERSION}\n"
        return txt + "".join(f"{fmt(t[g])}\t{fmt(f32(m[g]))}\n" for g in range(len(t)))

    def select(self, sel):
        if sel[0] == "all":
            return np.arange(self.traj.n_atoms, dtype=np.int32)
        if sel[0] == "type_system":
            t = list(self.traj.type_names).index(sel[1])
            return np.nonzero(self.traj.types == t)[0].astype(np.int32)
        raise ValueError(sel)

    def name(self, p):
        return p.split("/")[-1]

    def times(self, s):
        return orc.displacement_times(s)

    def cmd_msd(self, a, lst):
        s = self.scheme()
        m = orc.msd(s, self.unwrapped, lst, self.mode)
        self.files[self.name(a[1])] = self.msd_text(m, s)

    def cmd_ngp(self, a, lst):
        s = self.scheme()
        q = orc.ngp(s, self.unwrapped, lst, self.mode)
        t = self.times(s)
        txt = f"Non-Gaussian parameter data created by AMDAT v.{VERSION}\n"
        txt += "".join(f"{fmt(t[g])}\t{fmt(f32(q[g]))}\n" for g in range(len(t)))
        self.files[self.name(a[1])] = txt

    def correlation_2d(self, sp, m0, m1, corr, s):
        approx = wv.approx_wavenumbers(sp)
        t = self.times(s)
        txt = f"Correlation data created by AMDAT v.{VERSION}\n\t"
        txt += "".join(fmt(approx[m]) + "\t" for m in range(m0, m1 + 1)) + "\n"
        for g in range(len(t)):
            txt += fmt(t[g]) + "\t" + "".join(fmt(f32(v)) + "\t" for v in corr[g]) + "\n"
        return txt

    def cmd_isfs(self, a, lst):
        m0, m1 = int(a[2]), int(a[3])
        maxlen = float(a[5])
        fb = int(a[6]) if len(a) > 6 else 0
        L = maxlen if maxlen > 0 else self.min_box()
        sp = wv.spacing(L)
        kv, off = self.shells(m0, m1)
        s = self.scheme()
        corr = orc.isfs(s, self.unwrapped, lst, kv, off, float(sp), L, fb, self.mode)
        self.files[self.name(a[1])] = self.correlation_2d(sp, m0, m1, corr, s)

    def cmd_isf(self, a, lst):
        fb = int(a[5])
        m0, m1 = int(a[6]), int(a[7])
        L = self.min_box()
        sp = wv.spacing(L)
        kv, off = self.shells(m0, m1)
        s = self.scheme()
        frames = np.arange(orc.n_timesteps(s), dtype=np.int32)
        rho = orc.rhok(self.wrapped, lst, frames, kv, float(sp), L, self.mode)
        corr = orc.isf(s, rho, rho, off, len(lst), fb, self.mode)
        self.files[self.name(a[1])] = self.correlation_2d(sp, m0, m1, corr, s)

    def cmd_vhs(self, a, lst):
        rmax, nb = float(a[2]), int(a[3])
        vmax = f32(rmax) if f32(rmax) != 0 else f32(f32(self.traj.box.min()) / f32(2))
        s = self.scheme()
        counts, w, corr = orc.vhs(s, self.unwrapped, lst, float(vmax), nb)
        bs = f32(vmax / f32(nb))
        self.last_vhs = dict(corr=np.asarray(corr, np.float32), nb=nb, bs=bs)
        t = self.times(s)
        txt = f"Correlation data created by AMDAT v.{VERSION}\n{nb} bins\n{len(t)} times\n\n\t"
        txt += "".join(fmt(f32(f32(bs / f32(2)) + f32(f32(b) * bs))) + "\t" for b in range(nb)) + "\n"
        for g in range(len(t)):
            vals = [fmt(f32(v)) for v in corr[g]]
            txt += fmt(t[g]) + "\t" + "".join(v + "\t" for v in vals[:-1]) + vals[-1] + "\n"
        self.files[self.name(a[1])] = txt

    def sk_shells(self, a):
        maxlen = float(a[4])
        ts = int(a[5])
        L = maxlen if maxlen > 0 else self.min_box()
        sp = wv.spacing(L)
        kv, off = self.shells(0, 98)
        return kv, off, sp, L, ts

    def cmd_structure_factor(self, a, lst):
        kv, off, sp, L, ts = self.sk_shells(a)
        s = self.scheme()
        S = orc.structure_factor(s, ts, self.wrapped, lst, kv, off, float(sp), L, self.mode)
        self.files[self.name(a[1])] = self.sk_text(S, kv, off, sp)

    def sk_text(self, S, kv, off, sp):
        approx = wv.approx_wavenumbers(sp)
        txt = (f"Structure factor data created by AMDAT v.{VERSION}\n"
               "Nominal_q\tMean_q\tStddev_q\tMean_qx\tMean_qy\tMean_qz\tS(q)\n")
        for m in range(99):
            vecs = wv.shell_vectors(kv[off[m]:off[m + 1]], sp)
            mv = wv.mean_wavevector(vecs)
            txt += "\t".join([fmt(approx[m]), fmt(wv.mean_wavenumber(vecs)),
                              fmt(wv.stdev_wavenumber(vecs)), fmt(mv[0]), fmt(mv[1]), fmt(mv[2]),
                              fmt(f32(S[m]))]) + "\n"
        txt += "\n"
        return txt

    def cmd_rdf(self, a, lst):
        nb, ts, maxlen = int(a[3]), int(a[4]), float(a[5])
        minbox = f32(self.traj.box.min())
        maxd = f32(maxlen) if (f32(maxlen) > 0 and f32(maxlen) < f32(minbox / f32(2))) \
            else f32(minbox / f32(2))
        s = self.scheme()
        counts, mean = orc.rdf(s, ts, self.wrapped, self.traj.box, lst, nb, float(maxd))
        bs = f32(maxd / f32(nb))
        if "s" in self.flags:
            frames = len(onetime := orc_frames(s, ts))
            self.stored[self.flags["s"]] = dict(mean=np.asarray(mean, np.float32), nb=nb, bs=bs, maxd=maxd,
                                                nj=len(lst), n_times=frames,
                                                vol=f32(f32(self.traj.box[0]) * f32(self.traj.box[1])
                                                        * f32(self.traj.box[2])))
        txt = f"Radial distribution function data created by AMDAT v.{VERSION}\n"
        txt += "".join(fmt(f32(f32(f32(b) * bs) + f32(bs / f32(2)))) + "\t" for b in range(nb)) + "\n"
        txt += "".join(fmt(f32(v)) + "\t" for v in mean) + "\n"
        self.files[self.name(a[1])] = txt

    def cmd_msd_2d(self, a, lst):
        plane = {"xy": 0, "xz": 1, "yz": 2}[a[2]]
        s = self.scheme()
        m = orc.msd2d(s, self.unwrapped, lst, plane, self.mode)
        self.files[self.name(a[1])] = self.msd2d_text(a[2], m, s)

    def cmd_mean_displacement(self, a, lst):
        s = self.scheme()
        md = orc.mean_disp(s, self.unwrapped, lst, self.mode)
        self.files[self.name(a[1])] = self.md_text(md, s)

    def _u2(self, lst, bins, maxvalue, gap):
        s = self.scheme()
        mean, var, dist = orc.u2dist(s, self.unwrapped, lst, gap, bins, maxvalue, self.mode)
        bs = f32(f32(maxvalue) / f32(bins))
        rows = "".join(f"{fmt((float(f32(b)) + 0.5) * float(bs))}\t{fmt(f32(d))}\n" for b, d in enumerate(dist))
        return fmt(self.times(s)[gap]), fmt(f32(mean)), fmt(f32(var)), rows

    def cmd_u2dist(self, a, lst):
        t, mean, var, rows = self._u2(lst, int(a[2]), float(a[3]), int(a[4]))
        txt = (f"MSD distribution created by AMDAT v.{VERSION}\nMSD time = {t}\n"
               f"Mean_stiffness\t{mean}\nVariance\t{var}\n\n" + rows + "Last bin includes overflow.")
        self.files[self.name(a[1])] = txt

    def cmd_displacement_dist(self, a, lst):
        t, mean, var, rows = self._u2(lst, int(a[3]), float(a[4]), int(a[5]))
        txt = (f"Particle displacement distribution to the {fmt(f32(float(a[2])))} power created by "
               f"AMDAT v.{VERSION}\nLast bin includes overflow.time = {t}\nMean\t{mean}\n"
               f"Variance\t{var}\n\n" + rows)
        self.files[self.name(a[1])] = txt


def orc_frames(s, timescheme):
    """frames of Analysis_Onetime::analyze (as oracle.onetime_frames)"""
    return orc.onetime_frames(s, timescheme)


def _sk_from_rdf(st, n_ks):
    """Radial_Distribution_Function::structure_factor (radial_distribution_function.cpp:379-434), FP32"""
    PI = 3.1459265
    mean_rho = f32(0)
    for _ in range(st["n_times"]):
        mean_rho = f32(mean_rho + f32(f32(f32(st["nj"]) / st["vol"]) / f32(st["n_times"])))
    min_k = f32(2.0 * PI / float(st["maxd"]))
    ks, sk = [], []
    for k in range(n_ks):
        kk = f32(min_k * f32(k + 1))
        acc = f32(0)
        for b in range(st["nb"]):
            r = f32((float(f32(b)) + 0.5) * float(st["bs"]))
            term = f32(f32(f32(f32(st["mean"][b] - f32(1)) * r) * f32(np.sin(f32(kk * r)))) / kk)
            acc = f32(acc + f32(term * st["bs"]))
        ks.append(kk)
        sk.append(f32(1.0 + 4.0 * PI * float(mean_rho) * float(acc)))
    return ks, sk


def _cmd_sk_from_rdf(self, a):
    name, n_ks = a[3], int(a[2])
    if name not in self.stored:
        return
    ks, sk = _sk_from_rdf(self.stored[name], n_ks)
    txt = f"Structure factor data calculated from g(r) created by AMDAT v.{VERSION}\n"
    txt += "".join(fmt(k) + "\t" for k in ks) + "\n"
    txt += "".join(fmt(v) + "\t" for v in sk) + "\n"
    self.files[self.name(a[1])] = txt


OracleRun.cmd_structure_factor_from_rdf = _cmd_sk_from_rdf
