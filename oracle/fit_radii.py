"""CPU restatement of the reference's HBT radii fit
(ebe_scripts/fit_HBT_radii.py) for one correlation table - TEST
INFRASTRUCTURE ONLY (the oracle of the GPU fits and the timed CPU
comparison of the benchmark's fit leg; the product is hbt_fit_radii).

Per table (an eight-column array, :60-67): nan_to_num, columns 0-2 as
q_out, q_side, q_long, column 6 as C and column 7 + 1e-15 as its error;
for every q_cut in (0.05, 0.075, 0.1, 0.125, 0.15) (:37) the rows with
q_cut_min < |q| < q_cut (:71-72) are fitted with scipy's curve_fit from
p0 = (1, 5, 5, 5, 0.1, 0.1) with absolute sigma (:75-79) to
lambda exp(-((R_out q_out)^2 + (R_side q_side)^2 + (R_long q_long)^2
+ 2 q_out q_side R_os^2 + 2 q_out q_long R_ol^2)), radii in fm divided by
hbar c = 0.19733 (:13-29); a row is q_cut followed by each parameter and
sqrt of its covariance diagonal (:80-92).

Parity pin: over tests/golden_fit/ the rows equal those the unmodified
script stores (tests/golden_fit/make_golden_fit.py ran it).
"""
import numpy as np
from scipy.optimize import curve_fit

HBARC = 0.19733
EPS = 1e-15
Q_CUT_MAX_LIST = (0.05, 0.075, 0.1, 0.125, 0.15)
KT_CUT_LIST = ("0_0.2", "0.2_0.4", "0.4_0.6", "0.6_0.8")
P0 = (1.0, 5.0, 5.0, 5.0, 0.1, 0.1)
HEADER = ("# q_cut[GeV]  lambda  lambda_err  R_out[fm]  R_out_err[fm]  "
          "R_side[fm]  R_side_err[fm]  R_long [fm]  R_long_err[fm]  "
          "R_os[fm]  R_os_err[fm]  R_ol[fm]  R_ol_err[fm]")


def gaussian_3d(q_arr, lambda_, R_out, R_side, R_long, R_os, R_ol):
    q_out, q_side, q_long = q_arr
    R_out /= HBARC
    R_side /= HBARC
    R_long /= HBARC
    R_os /= HBARC
    R_ol /= HBARC
    gauss = lambda_ * np.exp(-((R_out * q_out) ** 2 + (R_side * q_side) ** 2
                               + (R_long * q_long) ** 2 + 2. * q_out * q_side * R_os ** 2.
                               + 2. * q_out * q_long * R_ol ** 2.))
    return np.ravel(gauss)


def fit_table(table, q_cut_max_list=Q_CUT_MAX_LIST, q_cut_min=0.0, p0=P0):
    """Rows [q_cut, lambda, lambda_err, R_out, R_out_err, ..., R_ol_err]."""
    data = np.nan_to_num(np.asarray(table, dtype=float))
    q_out, q_side, q_long = data[:, 0], data[:, 1], data[:, 2]
    corr, corr_err = data[:, 6], data[:, 7] + EPS
    q = np.sqrt(q_out ** 2. + q_side ** 2. + q_long ** 2.)
    rows = []
    for q_cut in q_cut_max_list:
        idx = (q > q_cut_min) & (q < q_cut)
        q_arr = [q_out[idx], q_side[idx], q_long[idx]]
        popt, pcov = curve_fit(gaussian_3d, q_arr, np.ravel(corr[idx]), p0=list(p0),
                               sigma=np.ravel(corr_err[idx]), absolute_sigma=True)
        perr = np.sqrt(np.diag(pcov))
        row = [q_cut]
        for x, e in zip(popt, perr):
            row += [x, e]
        rows.append(row)
    return np.array(rows)
