/*
 * pt_tableau.h -- Butcher tableaux of the two embedded Runge-Kutta methods.
 *
 * The coefficients are those of the published methods (Cash & Karp 1990;
 * Dormand & Prince 8(5,3) as distributed with Hairer's DOP853) with the exact
 * decimal forms the reference uses, so the compiled doubles are the same:
 *   Cash-Karp: sources/integrations.F90:86-98 (integers over a common
 *     denominator, divided at compile time);
 *   DOP853:    sources/integrations.F90:255-326.
 * Plain constexpr scalars: usable as immediates in device code and on the host.
 */
#ifndef PT_TABLEAU_H
#define PT_TABLEAU_H

namespace pt_tab {

/* ---- Cash-Karp RK5(4): stage j uses CK_Bj_i * k_i (k includes dt) ---- */
constexpr double CK_DEN = 5.5296e+05;
constexpr double CK_B2_1 = 1.10592e+05 / CK_DEN;
constexpr double CK_B3_1 = 4.14720e+04 / CK_DEN;
constexpr double CK_B3_2 = 1.24416e+05 / CK_DEN;
constexpr double CK_B4_1 = 1.65888e+05 / CK_DEN;
constexpr double CK_B4_2 = -4.97664e+05 / CK_DEN;
constexpr double CK_B4_3 = 6.63552e+05 / CK_DEN;
constexpr double CK_B5_1 = -1.12640e+05 / CK_DEN;
constexpr double CK_B5_2 = 1.38240e+06 / CK_DEN;
constexpr double CK_B5_3 = -1.43360e+06 / CK_DEN;
constexpr double CK_B5_4 = 7.16800e+05 / CK_DEN;
constexpr double CK_B6_1 = 1.63100e+04 / CK_DEN;
constexpr double CK_B6_2 = 1.89000e+05 / CK_DEN;
constexpr double CK_B6_3 = 2.30000e+04 / CK_DEN;
constexpr double CK_B6_4 = 2.21375e+05 / CK_DEN;
constexpr double CK_B6_5 = 3.41550e+04 / CK_DEN;
/* 5th-order weights c and error weights d = c - c* */
constexpr double CK_C1 = 9.361e+03 / 9.5634e+04;
constexpr double CK_C2 = 0.0 / 9.5634e+04;
constexpr double CK_C3 = 3.85e+04 / 9.5634e+04;
constexpr double CK_C4 = 2.0125e+04 / 9.5634e+04;
constexpr double CK_C5 = 0.0 / 9.5634e+04;
constexpr double CK_C6 = 2.7648e+04 / 9.5634e+04;
constexpr double CK_D1 = -1.40162e+05 / 3.2643072e+07;
constexpr double CK_D2 = 0.0 / 3.2643072e+07;
constexpr double CK_D3 = 6.094e+05 / 3.2643072e+07;
constexpr double CK_D4 = -1.114925e+06 / 3.2643072e+07;
constexpr double CK_D5 = -6.30729e+05 / 3.2643072e+07;
constexpr double CK_D6 = 1.276416e+06 / 3.2643072e+07;

/* ---- Dormand-Prince 8(5,3) ---- */
constexpr double A0201 = 5.26001519587677318785587544488e-02;
constexpr double A0301 = 1.97250569845378994544595329183e-02;
constexpr double A0302 = 5.91751709536136983633785987549e-02;
constexpr double A0401 = 2.95875854768068491816892993775e-02;
constexpr double A0403 = 8.87627564304205475450678981324e-02;
constexpr double A0501 = 2.41365134159266685502369798665e-01;
constexpr double A0503 = -8.84549479328286085344864962717e-01;
constexpr double A0504 = 9.24834003261792003115737966543e-01;
constexpr double A0601 = 3.70370370370370370370370370370e-02;
constexpr double A0604 = 1.70828608729473871279604482173e-01;
constexpr double A0605 = 1.25467687566822425016691814123e-01;
constexpr double A0701 = 3.71093750000000000000000000000e-02;
constexpr double A0704 = 1.70252211019544039314978060272e-01;
constexpr double A0705 = 6.02165389804559606850219397283e-02;
constexpr double A0706 = -1.75781250000000000000000000000e-02;
constexpr double A0801 = 3.70920001185047927108779319836e-02;
constexpr double A0804 = 1.70383925712239993810214054705e-01;
constexpr double A0805 = 1.07262030446373284651809199168e-01;
constexpr double A0806 = -1.53194377486244017527936158236e-02;
constexpr double A0807 = 8.27378916381402288758473766002e-03;
constexpr double A0901 = 6.24110958716075717114429577812e-01;
constexpr double A0904 = -3.36089262944694129406857109825e+00;
constexpr double A0905 = -8.68219346841726006818189891453e-01;
constexpr double A0906 = 2.75920996994467083049415600797e+01;
constexpr double A0907 = 2.01540675504778934086186788979e+01;
constexpr double A0908 = -4.34898841810699588477366255144e+01;
constexpr double A1001 = 4.77662536438264365890433908527e-01;
constexpr double A1004 = -2.48811461997166764192642586468e+00;
constexpr double A1005 = -5.90290826836842996371446475743e-01;
constexpr double A1006 = 2.12300514481811942347288949897e+01;
constexpr double A1007 = 1.52792336328824235832596922938e+01;
constexpr double A1008 = -3.32882109689848629194453265587e+01;
constexpr double A1009 = -2.03312017085086261358222928593e-02;
constexpr double A1101 = -9.37142430085987325717040216580e-01;
constexpr double A1104 = 5.18637242884406370830023853209e+00;
constexpr double A1105 = 1.09143734899672957818500254654e+00;
constexpr double A1106 = -8.14978701074692612513997267357e+00;
constexpr double A1107 = -1.85200656599969598641566180701e+01;
constexpr double A1108 = 2.27394870993505042818970056734e+01;
constexpr double A1109 = 2.49360555267965238987089396762e+00;
constexpr double A1110 = -3.04676447189821950038236690220e+00;
constexpr double A1201 = 2.27331014751653820792359768449e+00;
constexpr double A1204 = -1.05344954667372501984066689879e+01;
constexpr double A1205 = -2.00087205822486249909675718444e+00;
constexpr double A1206 = -1.79589318631187989172765950534e+01;
constexpr double A1207 = 2.79488845294199600508499808837e+01;
constexpr double A1208 = -2.85899827713502369474065508674e+00;
constexpr double A1209 = -8.87285693353062954433549289258e+00;
constexpr double A1210 = 1.23605671757943030647266201528e+01;
constexpr double A1211 = 6.43392746015763530355970484046e-01;

constexpr double B01 = 5.42937341165687622380535766363e-02;
constexpr double B06 = 4.45031289275240888144113950566e+00;
constexpr double B07 = 1.89151789931450038304281599044e+00;
constexpr double B08 = -5.80120396001058478146721142270e+00;
constexpr double B09 = 3.11164366957819894408916062370e-01;
constexpr double B10 = -1.52160949662516078556178806805e-01;
constexpr double B11 = 2.01365400804030348374776537501e-01;
constexpr double B12 = 4.47106157277725905176885569043e-02;

constexpr double BH1 = 0.244094488188976377952755905512e+00;
constexpr double BH2 = 0.733846688281611857341361741547e+00;
constexpr double BH3 = 0.220588235294117647058823529412e-01;

constexpr double ER01 = 0.1312004499419488073250102996e-01;
constexpr double ER06 = -0.1225156446376204440720569753e+01;
constexpr double ER07 = -0.4957589496572501915214079952e+00;
constexpr double ER08 = 0.1664377182454986536961530415e+01;
constexpr double ER09 = -0.3503288487499736816886487290e+00;
constexpr double ER10 = 0.3341791187130174790297318841e+00;
constexpr double ER11 = 0.8192320648511571246570742613e-01;
constexpr double ER12 = -0.2235530786388629525884427845e-01;

}  // namespace pt_tab

#endif /* PT_TABLEAU_H */
