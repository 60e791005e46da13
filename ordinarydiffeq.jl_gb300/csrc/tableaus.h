// Generated by gen_tableaus.py from the reference's Julia tableau sources; do not edit.
// Tsit5: lib/OrdinaryDiffEqTsit5/src/tsit_tableaus.jl:45-101,244-276
// Vern7: lib/OrdinaryDiffEqVerner/src/verner_tableaus.jl:648-716,880-972,1129-1205
// Rodas5P: lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_tableaus.jl:23-72
#pragma once
#include <cuda_runtime.h>
namespace odegb {
namespace tab {
// TSIT5
constexpr double TSIT5_c1 = 0.161;
constexpr double TSIT5_c2 = 0.327;
constexpr double TSIT5_c3 = 0.9;
constexpr double TSIT5_c4 = 0.9800255409045097;
constexpr double TSIT5_c5 = 1.0;
constexpr double TSIT5_c6 = 1.0;
constexpr double TSIT5_a21 = 0.161;
constexpr double TSIT5_a31 = -0.008480655492356989;
constexpr double TSIT5_a32 = 0.335480655492357;
constexpr double TSIT5_a41 = 2.8971530571054935;
constexpr double TSIT5_a42 = -6.359448489975075;
constexpr double TSIT5_a43 = 4.3622954328695815;
constexpr double TSIT5_a51 = 5.325864828439257;
constexpr double TSIT5_a52 = -11.748883564062828;
constexpr double TSIT5_a53 = 7.4955393428898365;
constexpr double TSIT5_a54 = -0.09249506636175525;
constexpr double TSIT5_a61 = 5.86145544294642;
constexpr double TSIT5_a62 = -12.92096931784711;
constexpr double TSIT5_a63 = 8.159367898576159;
constexpr double TSIT5_a64 = -0.071584973281401;
constexpr double TSIT5_a65 = -0.028269050394068383;
constexpr double TSIT5_a71 = 0.09646076681806523;
constexpr double TSIT5_a72 = 0.01;
constexpr double TSIT5_a73 = 0.4798896504144996;
constexpr double TSIT5_a74 = 1.379008574103742;
constexpr double TSIT5_a75 = -3.290069515436081;
constexpr double TSIT5_a76 = 2.324710524099774;
constexpr double TSIT5_btilde1 = -0.00178001105222577714;
constexpr double TSIT5_btilde2 = -0.0008164344596567469;
constexpr double TSIT5_btilde3 = 0.007880878010261995;
constexpr double TSIT5_btilde4 = -0.1447110071732629;
constexpr double TSIT5_btilde5 = 0.5823571654525552;
constexpr double TSIT5_btilde6 = -0.45808210592918697;
constexpr double TSIT5_btilde7 = 0.015151515151515152;
// TSIT5I
constexpr double TSIT5I_r11 = 1.0;
constexpr double TSIT5I_r12 = -2.763706197274826;
constexpr double TSIT5I_r13 = 2.9132554618219126;
constexpr double TSIT5I_r14 = -1.0530884977290216;
constexpr double TSIT5I_r22 = 0.13169999999999998;
constexpr double TSIT5I_r23 = -0.2234;
constexpr double TSIT5I_r24 = 0.1017;
constexpr double TSIT5I_r32 = 3.9302962368947516;
constexpr double TSIT5I_r33 = -5.941033872131505;
constexpr double TSIT5I_r34 = 2.490627285651253;
constexpr double TSIT5I_r42 = -12.411077166933676;
constexpr double TSIT5I_r43 = 30.33818863028232;
constexpr double TSIT5I_r44 = -16.548102889244902;
constexpr double TSIT5I_r52 = 37.50931341651104;
constexpr double TSIT5I_r53 = -88.1789048947664;
constexpr double TSIT5I_r54 = 47.37952196281928;
constexpr double TSIT5I_r62 = -27.896526289197286;
constexpr double TSIT5I_r63 = 65.09189467479366;
constexpr double TSIT5I_r64 = -34.87065786149661;
constexpr double TSIT5I_r72 = 1.5;
constexpr double TSIT5I_r73 = -4.0;
constexpr double TSIT5I_r74 = 2.5;
// VERN7
constexpr double VERN7_c2 = 0.005;
constexpr double VERN7_c3 = 0.10888888888888888;
constexpr double VERN7_c4 = 0.16333333333333333;
constexpr double VERN7_c5 = 0.4555;
constexpr double VERN7_c6 = 0.6095094489978381;
constexpr double VERN7_c7 = 0.884;
constexpr double VERN7_c8 = 0.925;
constexpr double VERN7_a021 = 0.005;
constexpr double VERN7_a031 = -1.07679012345679;
constexpr double VERN7_a032 = 1.185679012345679;
constexpr double VERN7_a041 = 0.04083333333333333;
constexpr double VERN7_a043 = 0.1225;
constexpr double VERN7_a051 = 0.6389139236255726;
constexpr double VERN7_a053 = -2.455672638223657;
constexpr double VERN7_a054 = 2.272258714598084;
constexpr double VERN7_a061 = -2.6615773750187572;
constexpr double VERN7_a063 = 10.804513886456137;
constexpr double VERN7_a064 = -8.3539146573962;
constexpr double VERN7_a065 = 0.820487594956657;
constexpr double VERN7_a071 = 6.067741434696772;
constexpr double VERN7_a073 = -24.711273635911088;
constexpr double VERN7_a074 = 20.427517930788895;
constexpr double VERN7_a075 = -1.9061579788166472;
constexpr double VERN7_a076 = 1.006172249242068;
constexpr double VERN7_a081 = 12.054670076253203;
constexpr double VERN7_a083 = -49.75478495046899;
constexpr double VERN7_a084 = 41.142888638604674;
constexpr double VERN7_a085 = -4.461760149974004;
constexpr double VERN7_a086 = 2.042334822239175;
constexpr double VERN7_a087 = -0.09834843665406107;
constexpr double VERN7_a091 = 10.138146522881808;
constexpr double VERN7_a093 = -42.6411360317175;
constexpr double VERN7_a094 = 35.76384003992257;
constexpr double VERN7_a095 = -4.3480228403929075;
constexpr double VERN7_a096 = 2.0098622683770357;
constexpr double VERN7_a097 = 0.3487490460338272;
constexpr double VERN7_a098 = -0.27143900510483127;
constexpr double VERN7_a101 = -45.030072034298676;
constexpr double VERN7_a103 = 187.3272437654589;
constexpr double VERN7_a104 = -154.02882369350186;
constexpr double VERN7_a105 = 18.56465306347536;
constexpr double VERN7_a106 = -7.141809679295079;
constexpr double VERN7_a107 = 1.3088085781613787;
constexpr double VERN7_b1 = 0.04715561848627222;
constexpr double VERN7_b4 = 0.25750564298434153;
constexpr double VERN7_b5 = 0.26216653977412624;
constexpr double VERN7_b6 = 0.15216092656738558;
constexpr double VERN7_b7 = 0.4939969170032485;
constexpr double VERN7_b8 = -0.29430311714032503;
constexpr double VERN7_b9 = 0.08131747232495111;
constexpr double VERN7_btilde1 = 0.002547011879931045;
constexpr double VERN7_btilde4 = -0.00965839487279575;
constexpr double VERN7_btilde5 = 0.04206470975639691;
constexpr double VERN7_btilde6 = -0.0666822437469301;
constexpr double VERN7_btilde7 = 0.2650097464621281;
constexpr double VERN7_btilde8 = -0.29430311714032503;
constexpr double VERN7_btilde9 = 0.08131747232495111;
constexpr double VERN7_btilde10 = -0.02029518466335628;
// VERN7X
constexpr double VERN7X_c11 = 1.0;
constexpr double VERN7X_a1101 = 0.04715561848627222;
constexpr double VERN7X_a1104 = 0.25750564298434153;
constexpr double VERN7X_a1105 = 0.2621665397741262;
constexpr double VERN7X_a1106 = 0.15216092656738558;
constexpr double VERN7X_a1107 = 0.49399691700324844;
constexpr double VERN7X_a1108 = -0.29430311714032503;
constexpr double VERN7X_a1109 = 0.0813174723249511;
constexpr double VERN7X_c12 = 0.29;
constexpr double VERN7X_a1201 = 0.0523222769159969;
constexpr double VERN7X_a1204 = 0.22495861826705715;
constexpr double VERN7X_a1205 = 0.017443709248776376;
constexpr double VERN7X_a1206 = -0.007669379876829393;
constexpr double VERN7X_a1207 = 0.03435896044073285;
constexpr double VERN7X_a1208 = -0.0410209723009395;
constexpr double VERN7X_a1209 = 0.025651133005205617;
constexpr double VERN7X_a1211 = -0.0160443457;
constexpr double VERN7X_c13 = 0.125;
constexpr double VERN7X_a1301 = 0.053053341257859085;
constexpr double VERN7X_a1304 = 0.12195301011401886;
constexpr double VERN7X_a1305 = 0.017746840737602496;
constexpr double VERN7X_a1306 = -0.0005928372667681495;
constexpr double VERN7X_a1307 = 0.008381833970853752;
constexpr double VERN7X_a1308 = -0.01293369259698612;
constexpr double VERN7X_a1309 = 0.009412056815253861;
constexpr double VERN7X_a1311 = -0.005353253107275676;
constexpr double VERN7X_a1312 = -0.06666729992455811;
constexpr double VERN7X_c14 = 0.25;
constexpr double VERN7X_a1401 = 0.03887903257436304;
constexpr double VERN7X_a1404 = -0.0024403203308301317;
constexpr double VERN7X_a1405 = -0.0013928917214672623;
constexpr double VERN7X_a1406 = -0.00047446291558680135;
constexpr double VERN7X_a1407 = 0.00039207932413159514;
constexpr double VERN7X_a1408 = -0.00040554733285128004;
constexpr double VERN7X_a1409 = 0.00019897093147716726;
constexpr double VERN7X_a1411 = -0.00010278198793179169;
constexpr double VERN7X_a1412 = 0.03385661513870267;
constexpr double VERN7X_a1413 = 0.1814893063199928;
constexpr double VERN7X_c15 = 0.53;
constexpr double VERN7X_a1501 = 0.05723681204690013;
constexpr double VERN7X_a1504 = 0.22265948066761182;
constexpr double VERN7X_a1505 = 0.12344864200186899;
constexpr double VERN7X_a1506 = 0.04006332526666491;
constexpr double VERN7X_a1507 = -0.05269894848581452;
constexpr double VERN7X_a1508 = 0.04765971214244523;
constexpr double VERN7X_a1509 = -0.02138895885042213;
constexpr double VERN7X_a1511 = 0.015193891064036402;
constexpr double VERN7X_a1512 = 0.12060546716289655;
constexpr double VERN7X_a1513 = -0.022779423016187374;
constexpr double VERN7X_c16 = 0.79;
constexpr double VERN7X_a1601 = 0.051372038802756814;
constexpr double VERN7X_a1604 = 0.5414214473439406;
constexpr double VERN7X_a1605 = 0.350399806692184;
constexpr double VERN7X_a1606 = 0.14193112269692182;
constexpr double VERN7X_a1607 = 0.10527377478429423;
constexpr double VERN7X_a1608 = -0.031081847805874016;
constexpr double VERN7X_a1609 = -0.007401883149519145;
constexpr double VERN7X_a1611 = -0.006377932504865363;
constexpr double VERN7X_a1612 = -0.17325495908361865;
constexpr double VERN7X_a1613 = -0.18228156777622026;
// VERN7I
constexpr double VERN7I_r011 = 1.0;
constexpr double VERN7I_r012 = -8.413387198332767;
constexpr double VERN7I_r013 = 33.675508884490895;
constexpr double VERN7I_r014 = -70.80159089484886;
constexpr double VERN7I_r015 = 80.64695108301298;
constexpr double VERN7I_r016 = -47.19413969837522;
constexpr double VERN7I_r017 = 11.133813442539243;
constexpr double VERN7I_r042 = 8.754921980674396;
constexpr double VERN7I_r043 = -88.4596828699771;
constexpr double VERN7I_r044 = 346.9017638429916;
constexpr double VERN7I_r045 = -629.2580030059837;
constexpr double VERN7I_r046 = 529.6773755604193;
constexpr double VERN7I_r047 = -167.35886986514018;
constexpr double VERN7I_r052 = 8.913387586637922;
constexpr double VERN7I_r053 = -90.06081846893218;
constexpr double VERN7I_r054 = 353.1807459217058;
constexpr double VERN7I_r055 = -640.6476819744374;
constexpr double VERN7I_r056 = 539.2646279047156;
constexpr double VERN7I_r057 = -170.38809442991547;
constexpr double VERN7I_r062 = 5.1733120298478;
constexpr double VERN7I_r063 = -52.271115900055385;
constexpr double VERN7I_r064 = 204.9853867374073;
constexpr double VERN7I_r065 = -371.8306118563603;
constexpr double VERN7I_r066 = 312.9880934374529;
constexpr double VERN7I_r067 = -98.89290352172495;
constexpr double VERN7I_r072 = 16.79537744079696;
constexpr double VERN7I_r073 = -169.70040000059728;
constexpr double VERN7I_r074 = 665.4937727009246;
constexpr double VERN7I_r075 = -1207.1638892336007;
constexpr double VERN7I_r076 = 1016.1291515818546;
constexpr double VERN7I_r077 = -321.06001557237494;
constexpr double VERN7I_r082 = -10.005997536098665;
constexpr double VERN7I_r083 = 101.1005433052275;
constexpr double VERN7I_r084 = -396.47391512378437;
constexpr double VERN7I_r085 = 719.1787707014183;
constexpr double VERN7I_r086 = -605.3681033918824;
constexpr double VERN7I_r087 = 191.27439892797935;
constexpr double VERN7I_r092 = 2.764708833638599;
constexpr double VERN7I_r093 = -27.934602637390462;
constexpr double VERN7I_r094 = 109.54779186137893;
constexpr double VERN7I_r095 = -198.7128113064482;
constexpr double VERN7I_r096 = 167.26633571640318;
constexpr double VERN7I_r097 = -52.85010499525706;
constexpr double VERN7I_r112 = -2.1696320280163506;
constexpr double VERN7I_r113 = 22.016696037569876;
constexpr double VERN7I_r114 = -86.90152427798948;
constexpr double VERN7I_r115 = 159.22388973861476;
constexpr double VERN7I_r116 = -135.9618306534588;
constexpr double VERN7I_r117 = 43.792401183280006;
constexpr double VERN7I_r122 = -4.890070188793804;
constexpr double VERN7I_r123 = 22.75407737425176;
constexpr double VERN7I_r124 = -30.78034218537731;
constexpr double VERN7I_r125 = -2.797194317207249;
constexpr double VERN7I_r126 = 31.369456637508403;
constexpr double VERN7I_r127 = -15.655927320381801;
constexpr double VERN7I_r132 = 10.862170929551967;
constexpr double VERN7I_r133 = -50.542971417827104;
constexpr double VERN7I_r134 = 68.37148040407511;
constexpr double VERN7I_r135 = 6.213326521632409;
constexpr double VERN7I_r136 = -69.68006323194157;
constexpr double VERN7I_r137 = 34.776056794509195;
constexpr double VERN7I_r142 = -11.37286691922923;
constexpr double VERN7I_r143 = 130.79058078246717;
constexpr double VERN7I_r144 = -488.65113677785604;
constexpr double VERN7I_r145 = 832.2148793276441;
constexpr double VERN7I_r146 = -664.7743368554426;
constexpr double VERN7I_r147 = 201.79288044241662;
constexpr double VERN7I_r152 = -5.919778732715007;
constexpr double VERN7I_r153 = 63.27679965889219;
constexpr double VERN7I_r154 = -265.432682088738;
constexpr double VERN7I_r155 = 520.1009254140611;
constexpr double VERN7I_r156 = -467.412109533902;
constexpr double VERN7I_r157 = 155.3868452824017;
constexpr double VERN7I_r162 = -10.492146197961823;
constexpr double VERN7I_r163 = 105.35538525188011;
constexpr double VERN7I_r164 = -409.43975011988937;
constexpr double VERN7I_r165 = 732.831448907654;
constexpr double VERN7I_r166 = -606.3044574733512;
constexpr double VERN7I_r167 = 188.0495196316683;
// RODAS5P (8 stages): A lower triangular 8x8, C 8x7, c 8, d 8, H 3x8.
// Accessors are constexpr functions so device code folds them to immediates.
constexpr double RODAS5P_GAMMA = 0.21193756319429014;
__host__ __device__ constexpr double RODAS5P_A(int i, int j) {
    constexpr double t[8][8] = {{0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {3.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {2.849394379747939, 0.45842242204463923, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {-6.954028509809101, 2.489845061869568, -10.358996098473584, 0.0, 0.0, 0.0, 0.0, 0.0}, {2.8029986275628964, 0.5072464736228206, -0.3988312541770524, -0.04721187230404641, 0.0, 0.0, 0.0, 0.0}, {-7.502846399306121, 2.561846144803919, -11.627539656261098, -0.18268767659942256, 0.030198172008377946, 0.0, 0.0, 0.0}, {-7.502846399306121, 2.561846144803919, -11.627539656261098, -0.18268767659942256, 0.030198172008377946, 1.0, 0.0, 0.0}, {-7.502846399306121, 2.561846144803919, -11.627539656261098, -0.18268767659942256, 0.030198172008377946, 1.0, 1.0, 0.0}};
    return t[i][j];
}
__host__ __device__ constexpr double RODAS5P_C(int i, int j) {
    constexpr double t[8][7] = {{0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {-14.155112264123755, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {-17.97296035885952, -2.859693295451294, 0.0, 0.0, 0.0, 0.0, 0.0}, {147.12150275711716, -1.41221402718213, 71.68940251302358, 0.0, 0.0, 0.0, 0.0}, {165.43517024871676, -0.4592823456491126, 42.90938336958603, -5.961986721573306, 0.0, 0.0, 0.0}, {24.854864614690072, -3.0009227002832186, 47.4931110020768, 5.5814197821558125, -0.6610691825249471, 0.0, 0.0}, {30.91273214028599, -3.1208243349937974, 77.79954646070892, 34.28646028294783, -19.097331116725623, -28.087943162872662, 0.0}, {37.80277123390563, -3.2571969029072276, 112.26918849496327, 66.9347231244047, -40.06618937091002, -54.66780262877968, -9.48861652309627}};
    return t[i][j];
}
__host__ __device__ constexpr double RODAS5P_c(int i) {
    constexpr double t[8] = {0.0, 0.6358126895828704, 0.4095798393397535, 0.9769306725060716, 0.4288403609558664, 1.0, 1.0, 1.0};
    return t[i];
}
__host__ __device__ constexpr double RODAS5P_d(int i) {
    constexpr double t[8] = {0.21193756319429014, -0.42387512638858027, -0.3384627126235924, 1.8046452872882734, 2.325825639765069, 0.0, 0.0, 0.0};
    return t[i];
}
__host__ __device__ constexpr double RODAS5P_H(int i, int j) {
    constexpr double t[3][8] = {{25.948786856663858, -2.5579724845846235, 10.433815404888879, -2.3679251022685204, 0.524948541321073, 1.1241088310450404, 0.4272876194431874, -0.17202221070155493}, {-9.91568850695171, -0.9689944594115154, 3.0438037242978453, -24.495224566215796, 20.176138334709044, 15.98066361424651, -6.789040303419874, -6.710236069923372}, {11.419903575922262, 2.8879645146136994, 72.92137995996029, 80.12511834622643, -52.072871366152654, -59.78993625266729, -0.15582684282751913, 4.883087185713722}};
    return t[i][j];
}
__host__ __device__ constexpr double TSIT5_A(int i, int j) {
    constexpr double t[8][8] = {{0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.161, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, -0.008480655492356989, 0.335480655492357, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 2.8971530571054935, -6.359448489975075, 4.3622954328695815, 0.0, 0.0, 0.0, 0.0}, {0.0, 5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0.0, 0.0, 0.0}, {0.0, 5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383, 0.0, 0.0}, {0.0, 0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774, 0.0}};
    return t[i][j];
}
__host__ __device__ constexpr bool TSIT5_AM(int i, int j) {
    constexpr bool t[8][8] = {{false, false, false, false, false, false, false, false}, {false, false, false, false, false, false, false, false}, {false, true, false, false, false, false, false, false}, {false, true, true, false, false, false, false, false}, {false, true, true, true, false, false, false, false}, {false, true, true, true, true, false, false, false}, {false, true, true, true, true, true, false, false}, {false, true, true, true, true, true, true, false}};
    return t[i][j];
}
__host__ __device__ constexpr double TSIT5_CS(int i) {
    constexpr double t[8] = {0.0, 0.0, 0.161, 0.327, 0.9, 0.9800255409045097, 1.0, 1.0};
    return t[i];
}
__host__ __device__ constexpr double TSIT5_BT(int i) {
    constexpr double t[8] = {0.0, -0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995, -0.1447110071732629, 0.5823571654525552, -0.45808210592918697, 0.015151515151515152};
    return t[i];
}
__host__ __device__ constexpr double TSIT5_R(int i, int j) {
    constexpr double t[8][5] = {{0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 1.0, -2.763706197274826, 2.9132554618219126, -1.0530884977290216}, {0.0, 0.0, 0.13169999999999998, -0.2234, 0.1017}, {0.0, 0.0, 3.9302962368947516, -5.941033872131505, 2.490627285651253}, {0.0, 0.0, -12.411077166933676, 30.33818863028232, -16.548102889244902}, {0.0, 0.0, 37.50931341651104, -88.1789048947664, 47.37952196281928}, {0.0, 0.0, -27.896526289197286, 65.09189467479366, -34.87065786149661}, {0.0, 0.0, 1.5, -4.0, 2.5}};
    return t[i][j];
}
__host__ __device__ constexpr double VERN7_A(int i, int j) {
    constexpr double t[17][17] = {{0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.005, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, -1.07679012345679, 1.185679012345679, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.04083333333333333, 0.0, 0.1225, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.6389139236255726, 0.0, -2.455672638223657, 2.272258714598084, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, -2.6615773750187572, 0.0, 10.804513886456137, -8.3539146573962, 0.820487594956657, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 6.067741434696772, 0.0, -24.711273635911088, 20.427517930788895, -1.9061579788166472, 1.006172249242068, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 12.054670076253203, 0.0, -49.75478495046899, 41.142888638604674, -4.461760149974004, 2.042334822239175, -0.09834843665406107, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 10.138146522881808, 0.0, -42.6411360317175, 35.76384003992257, -4.3480228403929075, 2.0098622683770357, 0.3487490460338272, -0.27143900510483127, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, -45.030072034298676, 0.0, 187.3272437654589, -154.02882369350186, 18.56465306347536, -7.141809679295079, 1.3088085781613787, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.04715561848627222, 0.0, 0.0, 0.25750564298434153, 0.2621665397741262, 0.15216092656738558, 0.49399691700324844, -0.29430311714032503, 0.0813174723249511, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.0523222769159969, 0.0, 0.0, 0.22495861826705715, 0.017443709248776376, -0.007669379876829393, 0.03435896044073285, -0.0410209723009395, 0.025651133005205617, 0.0, -0.0160443457, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.053053341257859085, 0.0, 0.0, 0.12195301011401886, 0.017746840737602496, -0.0005928372667681495, 0.008381833970853752, -0.01293369259698612, 0.009412056815253861, 0.0, -0.005353253107275676, -0.06666729992455811, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.03887903257436304, 0.0, 0.0, -0.0024403203308301317, -0.0013928917214672623, -0.00047446291558680135, 0.00039207932413159514, -0.00040554733285128004, 0.00019897093147716726, 0.0, -0.00010278198793179169, 0.03385661513870267, 0.1814893063199928, 0.0, 0.0, 0.0}, {0.0, 0.05723681204690013, 0.0, 0.0, 0.22265948066761182, 0.12344864200186899, 0.04006332526666491, -0.05269894848581452, 0.04765971214244523, -0.02138895885042213, 0.0, 0.015193891064036402, 0.12060546716289655, -0.022779423016187374, 0.0, 0.0, 0.0}, {0.0, 0.051372038802756814, 0.0, 0.0, 0.5414214473439406, 0.350399806692184, 0.14193112269692182, 0.10527377478429423, -0.031081847805874016, -0.007401883149519145, 0.0, -0.006377932504865363, -0.17325495908361865, -0.18228156777622026, 0.0, 0.0, 0.0}};
    return t[i][j];
}
__host__ __device__ constexpr bool VERN7_AM(int i, int j) {
    constexpr bool t[17][17] = {{false, false, false, false, false, false, false, false, false, false, false, false, false, false, false, false, false}, {false, false, false, false, false, false, false, false, false, false, false, false, false, false, false, false, false}, {false, true, false, false, false, false, false, false, false, false, false, false, false, false, false, false, false}, {false, true, true, false, false, false, false, false, false, false, false, false, false, false, false, false, false}, {false, true, false, true, false, false, false, false, false, false, false, false, false, false, false, false, false}, {false, true, false, true, true, false, false, false, false, false, false, false, false, false, false, false, false}, {false, true, false, true, true, true, false, false, false, false, false, false, false, false, false, false, false}, {false, true, false, true, true, true, true, false, false, false, false, false, false, false, false, false, false}, {false, true, false, true, true, true, true, true, false, false, false, false, false, false, false, false, false}, {false, true, false, true, true, true, true, true, true, false, false, false, false, false, false, false, false}, {false, true, false, true, true, true, true, true, false, false, false, false, false, false, false, false, false}, {false, true, false, false, true, true, true, true, true, true, false, false, false, false, false, false, false}, {false, true, false, false, true, true, true, true, true, true, false, true, false, false, false, false, false}, {false, true, false, false, true, true, true, true, true, true, false, true, true, false, false, false, false}, {false, true, false, false, true, true, true, true, true, true, false, true, true, true, false, false, false}, {false, true, false, false, true, true, true, true, true, true, false, true, true, true, false, false, false}, {false, true, false, false, true, true, true, true, true, true, false, true, true, true, false, false, false}};
    return t[i][j];
}
__host__ __device__ constexpr double VERN7_CS(int i) {
    constexpr double t[17] = {0.0, 0.0, 0.005, 0.10888888888888888, 0.16333333333333333, 0.4555, 0.6095094489978381, 0.884, 0.925, 1.0, 1.0, 1.0, 0.29, 0.125, 0.25, 0.53, 0.79};
    return t[i];
}
__host__ __device__ constexpr double VERN7_B(int i) {
    constexpr double t[17] = {0.0, 0.04715561848627222, 0.0, 0.0, 0.25750564298434153, 0.26216653977412624, 0.15216092656738558, 0.4939969170032485, -0.29430311714032503, 0.08131747232495111, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    return t[i];
}
__host__ __device__ constexpr double VERN7_BT(int i) {
    constexpr double t[17] = {0.0, 0.002547011879931045, 0.0, 0.0, -0.00965839487279575, 0.04206470975639691, -0.0666822437469301, 0.2650097464621281, -0.29430311714032503, 0.08131747232495111, -0.02029518466335628, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    return t[i];
}
__host__ __device__ constexpr bool VERN7_BM(int j) {
    constexpr bool t[17] = {false, true, false, false, true, true, true, true, true, true, false, false, false, false, false, false, false};
    return t[j];
}
__host__ __device__ constexpr bool VERN7_BTM(int j) {
    constexpr bool t[17] = {false, true, false, false, true, true, true, true, true, true, true, false, false, false, false, false, false};
    return t[j];
}
__host__ __device__ constexpr double VERN7_R(int i, int j) {
    constexpr double t[17][8] = {{0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 1.0, -8.413387198332767, 33.675508884490895, -70.80159089484886, 80.64695108301298, -47.19413969837522, 11.133813442539243}, {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 8.754921980674396, -88.4596828699771, 346.9017638429916, -629.2580030059837, 529.6773755604193, -167.35886986514018}, {0.0, 0.0, 8.913387586637922, -90.06081846893218, 353.1807459217058, -640.6476819744374, 539.2646279047156, -170.38809442991547}, {0.0, 0.0, 5.1733120298478, -52.271115900055385, 204.9853867374073, -371.8306118563603, 312.9880934374529, -98.89290352172495}, {0.0, 0.0, 16.79537744079696, -169.70040000059728, 665.4937727009246, -1207.1638892336007, 1016.1291515818546, -321.06001557237494}, {0.0, 0.0, -10.005997536098665, 101.1005433052275, -396.47391512378437, 719.1787707014183, -605.3681033918824, 191.27439892797935}, {0.0, 0.0, 2.764708833638599, -27.934602637390462, 109.54779186137893, -198.7128113064482, 167.26633571640318, -52.85010499525706}, {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, -2.1696320280163506, 22.016696037569876, -86.90152427798948, 159.22388973861476, -135.9618306534588, 43.792401183280006}, {0.0, 0.0, -4.890070188793804, 22.75407737425176, -30.78034218537731, -2.797194317207249, 31.369456637508403, -15.655927320381801}, {0.0, 0.0, 10.862170929551967, -50.542971417827104, 68.37148040407511, 6.213326521632409, -69.68006323194157, 34.776056794509195}, {0.0, 0.0, -11.37286691922923, 130.79058078246717, -488.65113677785604, 832.2148793276441, -664.7743368554426, 201.79288044241662}, {0.0, 0.0, -5.919778732715007, 63.27679965889219, -265.432682088738, 520.1009254140611, -467.412109533902, 155.3868452824017}, {0.0, 0.0, -10.492146197961823, 105.35538525188011, -409.43975011988937, 732.831448907654, -606.3044574733512, 188.0495196316683}};
    return t[i][j];
}
}  // namespace tab
}  // namespace odegb
