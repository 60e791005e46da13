// Generated by gen_tableaus.py from the reference's Julia tableau sources; do not edit.
// Tsit5: lib/OrdinaryDiffEqTsit5/src/tsit_tableaus.jl:45-101,244-276
// Vern7: lib/OrdinaryDiffEqVerner/src/verner_tableaus.jl:648-716,880-972,1129-1205
// Rodas5P: lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_tableaus.jl:23-72
// Rosenbrock23: lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_tableaus.jl:6-10
#pragma once
#ifndef __CUDACC_RTC__
#include <cuda_runtime.h>
#endif
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
__host__ __device__ constexpr float RODAS5P_A_HI(int i, int j) {
    constexpr float t[8][8] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.8000000000000p+1f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.6cb8f40000000p+1f, 0x1.d56cb00000000p-2f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.bd0ece0000000p+2f, 0x1.3eb33e0000000p+1f, -0x1.4b7ce60000000p+3f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.66c8a80000000p+1f, 0x1.03b5d00000000p-1f, -0x1.9867380000000p-2f, -0x1.82c2780000000p-5f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.e02ea20000000p+2f, 0x1.47ea940000000p+1f, -0x1.7414ce0000000p+3f, -0x1.7624f40000000p-3f, 0x1.eec4500000000p-6f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.e02ea20000000p+2f, 0x1.47ea940000000p+1f, -0x1.7414ce0000000p+3f, -0x1.7624f40000000p-3f, 0x1.eec4500000000p-6f, 0x1.0000000000000p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.e02ea20000000p+2f, 0x1.47ea940000000p+1f, -0x1.7414ce0000000p+3f, -0x1.7624f40000000p-3f, 0x1.eec4500000000p-6f, 0x1.0000000000000p+0f, 0x1.0000000000000p+0f, 0x0.0p+0f}};
    return t[i][j];
}
__host__ __device__ constexpr float RODAS5P_A_LO(int i, int j) {
    constexpr float t[8][8] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.f4d8e20000000p-25f, -0x1.90aea80000000p-32f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.9eeb160000000p-24f, 0x1.a358fa0000000p-26f, 0x1.3a6a840000000p-22f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.6c1d940000000p-24f, -0x1.631d580000000p-26f, -0x1.9502780000000p-28f, -0x1.e1d7fc0000000p-30f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.53f7300000000p-23f, -0x1.deaef80000000p-24f, -0x1.7256860000000p-26f, -0x1.c607260000000p-28f, 0x1.2cca900000000p-32f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.53f7300000000p-23f, -0x1.deaef80000000p-24f, -0x1.7256860000000p-26f, -0x1.c607260000000p-28f, 0x1.2cca900000000p-32f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.53f7300000000p-23f, -0x1.deaef80000000p-24f, -0x1.7256860000000p-26f, -0x1.c607260000000p-28f, 0x1.2cca900000000p-32f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}};
    return t[i][j];
}
__host__ __device__ constexpr double RODAS5P_C(int i, int j) {
    constexpr double t[8][7] = {{0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {-14.155112264123755, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {-17.97296035885952, -2.859693295451294, 0.0, 0.0, 0.0, 0.0, 0.0}, {147.12150275711716, -1.41221402718213, 71.68940251302358, 0.0, 0.0, 0.0, 0.0}, {165.43517024871676, -0.4592823456491126, 42.90938336958603, -5.961986721573306, 0.0, 0.0, 0.0}, {24.854864614690072, -3.0009227002832186, 47.4931110020768, 5.5814197821558125, -0.6610691825249471, 0.0, 0.0}, {30.91273214028599, -3.1208243349937974, 77.79954646070892, 34.28646028294783, -19.097331116725623, -28.087943162872662, 0.0}, {37.80277123390563, -3.2571969029072276, 112.26918849496327, 66.9347231244047, -40.06618937091002, -54.66780262877968, -9.48861652309627}};
    return t[i][j];
}
__host__ __device__ constexpr float RODAS5P_C_HI(int i, int j) {
    constexpr float t[8][7] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.c4f6ae0000000p+3f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.1f913e0000000p+4f, -0x1.6e0a6e0000000p+1f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.263e360000000p+7f, -0x1.6986dc0000000p+0f, 0x1.1ec1f20000000p+6f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.4adece0000000p+7f, -0x1.d64e1c0000000p-2f, 0x1.57466a0000000p+5f, -0x1.7d91300000000p+2f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.8dad860000000p+4f, -0x1.801e3c0000000p+1f, 0x1.7bf1e40000000p+5f, 0x1.6535fc0000000p+2f, -0x1.5277a80000000p-1f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.ee9a8e0000000p+4f, -0x1.8f772c0000000p+1f, 0x1.3732bc0000000p+6f, 0x1.124aac0000000p+5f, -0x1.318eac0000000p+4f, -0x1.c168380000000p+4f, 0x0.0p+0f}, {0x1.2e6c140000000p+5f, -0x1.a0ebd40000000p+1f, 0x1.c113a60000000p+6f, 0x1.0bbd280000000p+6f, -0x1.40878e0000000p+5f, -0x1.b557a80000000p+5f, -0x1.2fa2c00000000p+3f}};
    return t[i][j];
}
__host__ __device__ constexpr float RODAS5P_C_LO(int i, int j) {
    constexpr float t[8][7] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.4c28a00000000p-29f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.c333640000000p-21f, -0x1.c8dc420000000p-28f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.8ffe760000000p-19f, 0x1.d267020000000p-27f, 0x1.76f9bc0000000p-19f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.4509b80000000p-18f, -0x1.e316f60000000p-28f, 0x1.937e600000000p-20f, -0x1.822bfc0000000p-23f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.0953400000000p-21f, -0x1.5e29680000000p-26f, 0x1.72cdee0000000p-22f, -0x1.5d32580000000p-23f, -0x1.dd5a380000000p-26f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.f76ed60000000p-21f, 0x1.14808c0000000p-29f, 0x1.3ac60a0000000p-20f, -0x1.3ea45c0000000p-21f, 0x1.da98f80000000p-21f, 0x1.d1f1c40000000p-21f, 0x0.0p+0f}, {-0x1.59c34a0000000p-20f, 0x1.6187400000000p-32f, 0x1.30ca740000000p-21f, 0x1.e1110a0000000p-23f, -0x1.2becd80000000p-21f, -0x1.cf2caa0000000p-20f, 0x1.c3410a0000000p-22f}};
    return t[i][j];
}
__host__ __device__ constexpr double RODAS5P_c(int i) {
    constexpr double t[8] = {0.0, 0.6358126895828704, 0.4095798393397535, 0.9769306725060716, 0.4288403609558664, 1.0, 1.0, 1.0};
    return t[i];
}
__host__ __device__ constexpr float RODAS5P_c_HI(int i) {
    constexpr float t[8] = {0x0.0p+0f, 0x1.45893e0000000p-1f, 0x1.a368e60000000p-2f, 0x1.f430420000000p-1f, 0x1.b721ee0000000p-2f, 0x1.0000000000000p+0f, 0x1.0000000000000p+0f, 0x1.0000000000000p+0f};
    return t[i];
}
__host__ __device__ constexpr float RODAS5P_c_LO(int i) {
    constexpr float t[8] = {0x0.0p+0f, -0x1.5ee0d00000000p-27f, -0x1.0ef50a0000000p-28f, -0x1.7208c00000000p-28f, -0x1.13eaf20000000p-27f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f};
    return t[i];
}
__host__ __device__ constexpr double RODAS5P_d(int i) {
    constexpr double t[8] = {0.21193756319429014, -0.42387512638858027, -0.3384627126235924, 1.8046452872882734, 2.325825639765069, 0.0, 0.0, 0.0};
    return t[i];
}
__host__ __device__ constexpr float RODAS5P_d_HI(int i) {
    constexpr float t[8] = {0x1.b20c520000000p-3f, -0x1.b20c520000000p-2f, -0x1.5a95f80000000p-2f, 0x1.cdfd3c0000000p+0f, 0x1.29b4a80000000p+1f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f};
    return t[i];
}
__host__ __device__ constexpr float RODAS5P_d_LO(int i) {
    constexpr float t[8] = {0x1.ada8800000000p-30f, -0x1.ada8800000000p-29f, -0x1.3447e40000000p-29f, -0x1.b1bb100000000p-27f, -0x1.ba05820000000p-25f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f};
    return t[i];
}
__host__ __device__ constexpr double RODAS5P_H(int i, int j) {
    constexpr double t[3][8] = {{25.948786856663858, -2.5579724845846235, 10.433815404888879, -2.3679251022685204, 0.524948541321073, 1.1241088310450404, 0.4272876194431874, -0.17202221070155493}, {-9.91568850695171, -0.9689944594115154, 3.0438037242978453, -24.495224566215796, 20.176138334709044, 15.98066361424651, -6.789040303419874, -6.710236069923372}, {11.419903575922262, 2.8879645146136994, 72.92137995996029, 80.12511834622643, -52.072871366152654, -59.78993625266729, -0.15582684282751913, 4.883087185713722}};
    return t[i][j];
}
__host__ __device__ constexpr float RODAS5P_H_HI(int i, int j) {
    constexpr float t[3][8] = {{0x1.9f2e3c0000000p+4f, -0x1.476ba40000000p+1f, 0x1.4de1d00000000p+3f, -0x1.2f182c0000000p+1f, 0x1.0cc60e0000000p-1f, 0x1.1fc5980000000p+0f, 0x1.b58ae20000000p-2f, -0x1.604d2e0000000p-3f}, {-0x1.3d4d520000000p+3f, -0x1.f0200a0000000p-1f, 0x1.859b5c0000000p+1f, -0x1.87ec700000000p+4f, 0x1.42d1760000000p+4f, 0x1.ff61980000000p+3f, -0x1.b27fa20000000p+2f, -0x1.ad74820000000p+2f}, {0x1.6d6fda0000000p+3f, 0x1.71a8d20000000p+1f, 0x1.23af7e0000000p+6f, 0x1.4080200000000p+6f, -0x1.a0953e0000000p+5f, -0x1.de51ca0000000p+5f, -0x1.3f22240000000p-3f, 0x1.3884800000000p+2f}};
    return t[i][j];
}
__host__ __device__ constexpr float RODAS5P_H_LO(int i, int j) {
    constexpr float t[3][8] = {{-0x1.bef8220000000p-21f, -0x1.cab7b80000000p-25f, 0x1.b01fec0000000p-22f, 0x1.1661160000000p-24f, 0x1.10e91e0000000p-28f, 0x1.54f76c0000000p-25f, 0x1.7bf4160000000p-27f, -0x1.24c2f80000000p-29f}, {0x1.0a8e000000000p-27f, -0x1.64b5ec0000000p-26f, 0x1.169ac00000000p-25f, -0x1.3082540000000p-21f, 0x1.b8c96c0000000p-22f, 0x1.51e4380000000p-22f, -0x1.cd35080000000p-23f, 0x1.67aa600000000p-29f}, {-0x1.80f8600000000p-23f, 0x1.d918f00000000p-26f, 0x1.d367040000000p-21f, -0x1.f3d6a00000000p-19f, 0x1.ab31e80000000p-21f, -0x1.9190be0000000p-23f, -0x1.9c87b00000000p-28f, 0x1.d8a0e40000000p-26f}};
    return t[i][j];
}
__host__ __device__ constexpr double TSIT5_A(int i, int j) {
    constexpr double t[8][8] = {{0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.161, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, -0.008480655492356989, 0.335480655492357, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 2.8971530571054935, -6.359448489975075, 4.3622954328695815, 0.0, 0.0, 0.0, 0.0}, {0.0, 5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0.0, 0.0, 0.0}, {0.0, 5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383, 0.0, 0.0}, {0.0, 0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774, 0.0}};
    return t[i][j];
}
__host__ __device__ constexpr float TSIT5_A_HI(int i, int j) {
    constexpr float t[8][8] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.49ba5e0000000p-3f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.15e4e40000000p-7f, 0x1.57883e0000000p-2f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.72d5ea0000000p+1f, -0x1.9701340000000p+2f, 0x1.172fda0000000p+2f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.54daf80000000p+2f, -0x1.77f6da0000000p+3f, 0x1.dfb6ea0000000p+2f, -0x1.7adc1c0000000p-4f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.7722160000000p+2f, -0x1.9d78940000000p+3f, 0x1.05198a0000000p+3f, -0x1.2536480000000p-4f, -0x1.cf28fe0000000p-6f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.8b1a720000000p-4f, 0x1.47ae140000000p-7f, 0x1.eb68320000000p-2f, 0x1.6106b40000000p+0f, -0x1.a521000000000p+1f, 0x1.29901e0000000p+1f, 0x0.0p+0f}};
    return t[i][j];
}
__host__ __device__ constexpr float TSIT5_A_LO(int i, int j) {
    constexpr float t[8][8] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.a9fbe80000000p-30f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.fd02480000000p-32f, -0x1.4383d40000000p-28f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.6039ba0000000p-24f, -0x1.ea143e0000000p-25f, -0x1.a22ae00000000p-23f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.3a20640000000p-25f, -0x1.540a5a0000000p-22f, 0x1.4bcbee0000000p-23f, 0x1.5deacc0000000p-29f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.4d50700000000p-29f, -0x1.4b31740000000p-22f, 0x1.6a1aae0000000p-22f, -0x1.e41de80000000p-29f, 0x1.11893e0000000p-32f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.2b59120000000p-32f, 0x1.eb851e0000000p-33f, -0x1.6e3f300000000p-27f, 0x1.6d5bbc0000000p-25f, 0x1.15a2ae0000000p-24f, -0x1.6653100000000p-24f, 0x0.0p+0f}};
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
__host__ __device__ constexpr float TSIT5_CS_HI(int i) {
    constexpr float t[8] = {0x0.0p+0f, 0x0.0p+0f, 0x1.49ba5e0000000p-3f, 0x1.4ed9160000000p-2f, 0x1.cccccc0000000p-1f, 0x1.f5c5e80000000p-1f, 0x1.0000000000000p+0f, 0x1.0000000000000p+0f};
    return t[i];
}
__host__ __device__ constexpr float TSIT5_CS_LO(int i) {
    constexpr float t[8] = {0x0.0p+0f, 0x0.0p+0f, 0x1.a9fbe80000000p-30f, 0x1.0e56040000000p-27f, 0x1.99999a0000000p-26f, 0x1.7b6fc80000000p-27f, 0x0.0p+0f, 0x0.0p+0f};
    return t[i];
}
__host__ __device__ constexpr double TSIT5_BT(int i) {
    constexpr double t[8] = {0.0, -0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995, -0.1447110071732629, 0.5823571654525552, -0.45808210592918697, 0.015151515151515152};
    return t[i];
}
__host__ __device__ constexpr float TSIT5_BT_HI(int i) {
    constexpr float t[8] = {0x0.0p+0f, -0x1.d29e860000000p-10f, -0x1.ac0bfa0000000p-11f, 0x1.023d980000000p-7f, -0x1.285e3e0000000p-3f, 0x1.2a2ab80000000p-1f, -0x1.d5137a0000000p-2f, 0x1.f07c200000000p-7f};
    return t[i];
}
__host__ __device__ constexpr float TSIT5_BT_LO(int i) {
    constexpr float t[8] = {0x0.0p+0f, 0x1.f410500000000p-35f, -0x1.b6b51e0000000p-37f, 0x1.515e040000000p-32f, -0x1.32e2dc0000000p-28f, -0x1.7947cc0000000p-29f, 0x1.026bde0000000p-28f, -0x1.f07c200000000p-32f};
    return t[i];
}
__host__ __device__ constexpr double TSIT5_R(int i, int j) {
    constexpr double t[8][5] = {{0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 1.0, -2.763706197274826, 2.9132554618219126, -1.0530884977290216}, {0.0, 0.0, 0.13169999999999998, -0.2234, 0.1017}, {0.0, 0.0, 3.9302962368947516, -5.941033872131505, 2.490627285651253}, {0.0, 0.0, -12.411077166933676, 30.33818863028232, -16.548102889244902}, {0.0, 0.0, 37.50931341651104, -88.1789048947664, 47.37952196281928}, {0.0, 0.0, -27.896526289197286, 65.09189467479366, -34.87065786149661}, {0.0, 0.0, 1.5, -4.0, 2.5}};
    return t[i][j];
}
__host__ __device__ constexpr float TSIT5_R_HI(int i, int j) {
    constexpr float t[8][5] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.0000000000000p+0f, -0x1.61c1200000000p+1f, 0x1.74e58e0000000p+1f, -0x1.0d97360000000p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.0db8ba0000000p-3f, -0x1.c985f00000000p-3f, 0x1.a0902e0000000p-4f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.f713f20000000p+1f, -0x1.7c39e60000000p+2f, 0x1.3ecce00000000p+1f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.8d278c0000000p+3f, 0x1.e569380000000p+4f, -0x1.08c5080000000p+4f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.2c13120000000p+5f, -0x1.60b7320000000p+6f, 0x1.7b09420000000p+5f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.be582c0000000p+4f, 0x1.045e1a0000000p+6f, -0x1.16f71c0000000p+5f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.8000000000000p+0f, -0x1.0000000000000p+2f, 0x1.4000000000000p+1f}};
    return t[i][j];
}
__host__ __device__ constexpr float TSIT5_R_LO(int i, int j) {
    constexpr float t[8][5] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.579de60000000p-27f, 0x1.2b59120000000p-27f, 0x1.9ceb900000000p-25f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.8e21960000000p-28f, -0x1.bda5120000000p-29f, -0x1.ff2e480000000p-32f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.d21c120000000p-25f, -0x1.1277540000000p-25f, -0x1.b348a80000000p-29f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.64f8ce0000000p-22f, 0x1.ecbc440000000p-22f, 0x1.dbf6680000000p-22f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.d335440000000p-20f, -0x1.b080ee0000000p-19f, 0x1.9f26c20000000p-20f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.97c96e0000000p-25f, -0x1.73115a0000000p-20f, 0x1.0fedde0000000p-20f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}};
    return t[i][j];
}
__host__ __device__ constexpr double VERN7_A(int i, int j) {
    constexpr double t[17][17] = {{0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.005, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, -1.07679012345679, 1.185679012345679, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.04083333333333333, 0.0, 0.1225, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.6389139236255726, 0.0, -2.455672638223657, 2.272258714598084, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, -2.6615773750187572, 0.0, 10.804513886456137, -8.3539146573962, 0.820487594956657, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 6.067741434696772, 0.0, -24.711273635911088, 20.427517930788895, -1.9061579788166472, 1.006172249242068, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 12.054670076253203, 0.0, -49.75478495046899, 41.142888638604674, -4.461760149974004, 2.042334822239175, -0.09834843665406107, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 10.138146522881808, 0.0, -42.6411360317175, 35.76384003992257, -4.3480228403929075, 2.0098622683770357, 0.3487490460338272, -0.27143900510483127, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, -45.030072034298676, 0.0, 187.3272437654589, -154.02882369350186, 18.56465306347536, -7.141809679295079, 1.3088085781613787, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.04715561848627222, 0.0, 0.0, 0.25750564298434153, 0.2621665397741262, 0.15216092656738558, 0.49399691700324844, -0.29430311714032503, 0.0813174723249511, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.0523222769159969, 0.0, 0.0, 0.22495861826705715, 0.017443709248776376, -0.007669379876829393, 0.03435896044073285, -0.0410209723009395, 0.025651133005205617, 0.0, -0.0160443457, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.053053341257859085, 0.0, 0.0, 0.12195301011401886, 0.017746840737602496, -0.0005928372667681495, 0.008381833970853752, -0.01293369259698612, 0.009412056815253861, 0.0, -0.005353253107275676, -0.06666729992455811, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.03887903257436304, 0.0, 0.0, -0.0024403203308301317, -0.0013928917214672623, -0.00047446291558680135, 0.00039207932413159514, -0.00040554733285128004, 0.00019897093147716726, 0.0, -0.00010278198793179169, 0.03385661513870267, 0.1814893063199928, 0.0, 0.0, 0.0}, {0.0, 0.05723681204690013, 0.0, 0.0, 0.22265948066761182, 0.12344864200186899, 0.04006332526666491, -0.05269894848581452, 0.04765971214244523, -0.02138895885042213, 0.0, 0.015193891064036402, 0.12060546716289655, -0.022779423016187374, 0.0, 0.0, 0.0}, {0.0, 0.051372038802756814, 0.0, 0.0, 0.5414214473439406, 0.350399806692184, 0.14193112269692182, 0.10527377478429423, -0.031081847805874016, -0.007401883149519145, 0.0, -0.006377932504865363, -0.17325495908361865, -0.18228156777622026, 0.0, 0.0, 0.0}};
    return t[i][j];
}
__host__ __device__ constexpr float VERN7_A_HI(int i, int j) {
    constexpr float t[17][17] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.47ae140000000p-8f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.13a8840000000p+0f, 0x1.2f88a80000000p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.4e81b40000000p-5f, 0x0.0p+0f, 0x1.f5c2900000000p-4f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.471fba0000000p-1f, 0x0.0p+0f, -0x1.3a537c0000000p+1f, 0x1.22d9600000000p+1f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.54ae920000000p+1f, 0x0.0p+0f, 0x1.59be940000000p+3f, -0x1.0b53440000000p+3f, 0x1.a416f40000000p-1f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.8455e00000000p+2f, 0x0.0p+0f, -0x1.8b61600000000p+4f, 0x1.46d71e0000000p+4f, -0x1.e7f9f80000000p+0f, 0x1.0194820000000p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.81bfdc0000000p+3f, 0x0.0p+0f, -0x1.8e09cc0000000p+5f, 0x1.4924a20000000p+5f, -0x1.1d8d7a0000000p+2f, 0x1.056b3a0000000p+1f, -0x1.92d5d00000000p-4f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.446bb20000000p+3f, 0x0.0p+0f, -0x1.55210c0000000p+5f, 0x1.1e1c580000000p+5f, -0x1.1646020000000p+2f, 0x1.01432a0000000p+1f, 0x1.651e780000000p-2f, -0x1.15f41c0000000p-2f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.683d960000000p+5f, 0x0.0p+0f, 0x1.76a78c0000000p+7f, -0x1.340ec20000000p+7f, 0x1.2908d20000000p+4f, -0x1.c913680000000p+2f, 0x1.4f0e140000000p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.824c800000000p-5f, 0x0.0p+0f, 0x0.0p+0f, 0x1.07af900000000p-2f, 0x1.0c75620000000p-2f, 0x1.37a0260000000p-3f, 0x1.f9da540000000p-2f, -0x1.2d5dcc0000000p-2f, 0x1.4d138c0000000p-4f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.ac9fc40000000p-5f, 0x0.0p+0f, 0x0.0p+0f, 0x1.ccb71a0000000p-3f, 0x1.1dcc380000000p-6f, -0x1.f69ed80000000p-8f, 0x1.1977f60000000p-5f, -0x1.500b360000000p-5f, 0x1.a444a60000000p-6f, 0x0.0p+0f, -0x1.06dede0000000p-6f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.b29cec0000000p-5f, 0x0.0p+0f, 0x0.0p+0f, 0x1.f385000000000p-4f, 0x1.22c3a60000000p-6f, -0x1.36d1460000000p-11f, 0x1.12a7ec0000000p-7f, -0x1.a7cfae0000000p-7f, 0x1.346a0e0000000p-7f, 0x0.0p+0f, -0x1.5ed4b00000000p-8f, -0x1.1111bc0000000p-4f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.3e7f3e0000000p-5f, 0x0.0p+0f, 0x0.0p+0f, -0x1.3fdb900000000p-9f, -0x1.6d23620000000p-10f, -0x1.f182ac0000000p-12f, 0x1.9b1ffe0000000p-12f, -0x1.a93f480000000p-12f, 0x1.a145b40000000p-13f, 0x0.0p+0f, -0x1.af19520000000p-14f, 0x1.155a780000000p-5f, 0x1.73b0aa0000000p-3f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.d4e24c0000000p-5f, 0x0.0p+0f, 0x0.0p+0f, 0x1.c801b20000000p-3f, 0x1.f9a5480000000p-4f, 0x1.4832e20000000p-5f, -0x1.afb5b40000000p-5f, 0x1.866daa0000000p-5f, -0x1.5e6fcc0000000p-6f, 0x0.0p+0f, 0x1.f1df980000000p-7f, 0x1.ee00000000000p-4f, -0x1.7537d40000000p-6f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.a4d6fa0000000p-5f, 0x0.0p+0f, 0x0.0p+0f, 0x1.1535320000000p-1f, 0x1.66cf340000000p-2f, 0x1.22acc80000000p-3f, 0x1.af338e0000000p-4f, -0x1.fd3eb80000000p-6f, -0x1.e516fe0000000p-8f, 0x0.0p+0f, -0x1.a1fbf40000000p-8f, -0x1.62d37e0000000p-3f, -0x1.75500a0000000p-3f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}};
    return t[i][j];
}
__host__ __device__ constexpr float VERN7_A_LO(int i, int j) {
    constexpr float t[17][17] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.eb851e0000000p-34f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.f39c620000000p-26f, 0x1.cb28140000000p-25f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.d0369c0000000p-30f, 0x0.0p+0f, -0x1.47ae140000000p-29f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.911b220000000p-28f, 0x0.0p+0f, 0x1.b925b80000000p-24f, -0x1.79801e0000000p-25f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.7a855a0000000p-24f, 0x0.0p+0f, -0x1.80fc700000000p-25f, -0x1.a9c5de0000000p-22f, -0x1.938cc40000000p-26f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.5d36a80000000p-25f, 0x0.0p+0f, -0x1.db2fb00000000p-22f, -0x1.ea99dc0000000p-21f, -0x1.2037380000000p-27f, -0x1.aeb9a20000000p-25f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.149b0c0000000p-22f, 0x0.0p+0f, -0x1.625c700000000p-20f, 0x1.98dc6e0000000p-20f, -0x1.c6bc020000000p-24f, 0x1.d3ff360000000p-26f, 0x1.1ea8980000000p-29f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.06eab00000000p-23f, 0x0.0p+0f, 0x1.27be380000000p-23f, 0x1.55b5f00000000p-22f, 0x1.a2405e0000000p-24f, 0x1.6824cc0000000p-24f, 0x1.339fb00000000p-28f, 0x1.71ba500000000p-27f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.a07ac80000000p-21f, 0x0.0p+0f, 0x1.fab3ba0000000p-19f, 0x1.5587a00000000p-23f, -0x1.65b2600000000p-22f, -0x1.cf6a100000000p-23f, 0x1.bf6b480000000p-27f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.8ebfe40000000p-33f, 0x0.0p+0f, 0x0.0p+0f, -0x1.a6c6400000000p-27f, 0x1.537b9c0000000p-27f, -0x1.2a7f540000000p-30f, -0x1.495bb20000000p-30f, 0x1.18afb20000000p-29f, 0x1.8754600000000p-29f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.0d36ae0000000p-30f, 0x0.0p+0f, 0x0.0p+0f, 0x1.4690d40000000p-28f, 0x1.7d25920000000p-33f, 0x1.fcc22e0000000p-35f, 0x1.b570d00000000p-31f, -0x1.9ee3da0000000p-30f, 0x1.5cda300000000p-32f, 0x0.0p+0f, 0x1.f765640000000p-31f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.2d4ed00000000p-31f, 0x0.0p+0f, 0x0.0p+0f, -0x1.e95a240000000p-32f, -0x1.b65bce0000000p-31f, 0x1.3cf39e0000000p-36f, -0x1.36f55a0000000p-32f, 0x1.47888c0000000p-32f, 0x1.ad479c0000000p-35f, 0x0.0p+0f, 0x1.f43eaa0000000p-33f, 0x1.e390960000000p-29f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.4be72a0000000p-31f, 0x0.0p+0f, 0x0.0p+0f, -0x1.9f79d00000000p-39f, 0x1.c038960000000p-36f, 0x1.6ba4540000000p-37f, -0x1.b545b00000000p-44f, -0x1.02ac400000000p-37f, 0x1.2fe8860000000p-38f, 0x0.0p+0f, 0x1.249fc00000000p-40f, -0x1.39dc060000000p-32f, 0x1.66faa20000000p-29f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.0866a60000000p-30f, 0x0.0p+0f, 0x0.0p+0f, -0x1.8c6ca60000000p-29f, 0x1.0446c60000000p-29f, -0x1.af70780000000p-35f, -0x1.11ee2c0000000p-30f, -0x1.c0bb2a0000000p-30f, 0x1.3df0400000000p-32f, 0x0.0p+0f, 0x1.3811e40000000p-32f, -0x1.b4427a0000000p-30f, 0x1.8fd63e0000000p-31f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.5a73c80000000p-30f, 0x0.0p+0f, 0x0.0p+0f, -0x1.b9381a0000000p-26f, 0x1.f224260000000p-27f, 0x1.a449160000000p-28f, -0x1.0b32fc0000000p-30f, 0x1.656ba80000000p-35f, -0x1.cabcc00000000p-37f, 0x0.0p+0f, 0x1.e6eb8c0000000p-34f, -0x1.f224b40000000p-28f, 0x1.de67440000000p-31f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}};
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
__host__ __device__ constexpr float VERN7_CS_HI(int i) {
    constexpr float t[17] = {0x0.0p+0f, 0x0.0p+0f, 0x1.47ae140000000p-8f, 0x1.be02460000000p-4f, 0x1.4e81b40000000p-3f, 0x1.d26e980000000p-2f, 0x1.3811a00000000p-1f, 0x1.c49ba60000000p-1f, 0x1.d9999a0000000p-1f, 0x1.0000000000000p+0f, 0x1.0000000000000p+0f, 0x1.0000000000000p+0f, 0x1.28f5c20000000p-2f, 0x1.0000000000000p-3f, 0x1.0000000000000p-2f, 0x1.0f5c280000000p-1f, 0x1.947ae20000000p-1f};
    return t[i];
}
__host__ __device__ constexpr float VERN7_CS_LO(int i) {
    constexpr float t[17] = {0x0.0p+0f, 0x0.0p+0f, 0x1.eb851e0000000p-34f, 0x1.159e260000000p-29f, 0x1.d0369c0000000p-28f, -0x1.cac0840000000p-28f, -0x1.47ce240000000p-26f, -0x1.cac0840000000p-29f, -0x1.99999a0000000p-27f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x1.1eb8520000000p-27f, 0x0.0p+0f, 0x0.0p+0f, 0x1.eb851e0000000p-26f, -0x1.70a3d80000000p-26f};
    return t[i];
}
__host__ __device__ constexpr double VERN7_B(int i) {
    constexpr double t[17] = {0.0, 0.04715561848627222, 0.0, 0.0, 0.25750564298434153, 0.26216653977412624, 0.15216092656738558, 0.4939969170032485, -0.29430311714032503, 0.08131747232495111, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    return t[i];
}
__host__ __device__ constexpr float VERN7_B_HI(int i) {
    constexpr float t[17] = {0x0.0p+0f, 0x1.824c800000000p-5f, 0x0.0p+0f, 0x0.0p+0f, 0x1.07af900000000p-2f, 0x1.0c75620000000p-2f, 0x1.37a0260000000p-3f, 0x1.f9da540000000p-2f, -0x1.2d5dcc0000000p-2f, 0x1.4d138c0000000p-4f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f};
    return t[i];
}
__host__ __device__ constexpr float VERN7_B_LO(int i) {
    constexpr float t[17] = {0x0.0p+0f, -0x1.8ebfe40000000p-33f, 0x0.0p+0f, 0x0.0p+0f, -0x1.a6c6400000000p-27f, 0x1.537b9c0000000p-27f, -0x1.2a7f540000000p-30f, -0x1.495bb00000000p-30f, 0x1.18afb20000000p-29f, 0x1.8754600000000p-29f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f};
    return t[i];
}
__host__ __device__ constexpr double VERN7_BT(int i) {
    constexpr double t[17] = {0.0, 0.002547011879931045, 0.0, 0.0, -0.00965839487279575, 0.04206470975639691, -0.0666822437469301, 0.2650097464621281, -0.29430311714032503, 0.08131747232495111, -0.02029518466335628, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    return t[i];
}
__host__ __device__ constexpr float VERN7_BT_HI(int i) {
    constexpr float t[17] = {0x0.0p+0f, 0x1.4dd78a0000000p-9f, 0x0.0p+0f, 0x0.0p+0f, -0x1.3c7c7e0000000p-7f, 0x1.5898180000000p-5f, -0x1.1121660000000p-4f, 0x1.0f5eb80000000p-2f, -0x1.2d5dcc0000000p-2f, 0x1.4d138c0000000p-4f, -0x1.4c842c0000000p-6f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f};
    return t[i];
}
__host__ __device__ constexpr float VERN7_BT_LO(int i) {
    constexpr float t[17] = {0x0.0p+0f, -0x1.17ba940000000p-34f, 0x0.0p+0f, 0x0.0p+0f, 0x1.e3b5800000000p-32f, -0x1.d1f46c0000000p-30f, -0x1.03be2e0000000p-29f, -0x1.ee975e0000000p-27f, 0x1.18afb20000000p-29f, 0x1.8754600000000p-29f, -0x1.329c560000000p-31f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f};
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
__host__ __device__ constexpr float VERN7_R_HI(int i, int j) {
    constexpr float t[17][8] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.0000000000000p+0f, -0x1.0d3a780000000p+3f, 0x1.0d67720000000p+5f, -0x1.1b34d40000000p+6f, 0x1.42967a0000000p+6f, -0x1.798d9a0000000p+5f, 0x1.6448340000000p+3f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.1828520000000p+3f, -0x1.61d6b80000000p+6f, 0x1.5ae6da0000000p+8f, -0x1.3aa1060000000p+9f, 0x1.08d6b40000000p+9f, -0x1.4eb7be0000000p+7f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.1d3a780000000p+3f, -0x1.683e480000000p+6f, 0x1.612e460000000p+8f, -0x1.4052e80000000p+9f, 0x1.0da1e00000000p+9f, -0x1.54c6b40000000p+7f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.4b178c0000000p+2f, -0x1.a22b3e0000000p+5f, 0x1.99f8840000000p+7f, -0x1.73d4a20000000p+8f, 0x1.38fcf40000000p+8f, -0x1.8b92560000000p+6f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.0cb9de0000000p+4f, -0x1.53669a0000000p+7f, 0x1.4cbf340000000p+9f, -0x1.2dca7e0000000p+10f, 0x1.fc10880000000p+9f, -0x1.410f5e0000000p+8f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.4031220000000p+3f, 0x1.9466f40000000p+6f, -0x1.8c79520000000p+8f, 0x1.6796e20000000p+9f, -0x1.2eaf1e0000000p+9f, 0x1.7e8c7e0000000p+7f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.61e1fa0000000p+1f, -0x1.bef4220000000p+4f, 0x1.b630f00000000p+6f, -0x1.8d6cf60000000p+7f, 0x1.4e885e0000000p+7f, -0x1.a6cd040000000p+5f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.15b6800000000p+1f, 0x1.6044640000000p+4f, -0x1.5b9b2a0000000p+6f, 0x1.3e72a20000000p+7f, -0x1.0fec760000000p+7f, 0x1.5e56d60000000p+5f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.38f6e80000000p+2f, 0x1.6c10b40000000p+4f, -0x1.ec7c480000000p+4f, -0x1.660a760000000p+1f, 0x1.f5e94c0000000p+4f, -0x1.f4fd5c0000000p+3f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.5b96e80000000p+3f, -0x1.9458020000000p+5f, 0x1.117c660000000p+6f, 0x1.8da7240000000p+2f, -0x1.16b8620000000p+6f, 0x1.16355e0000000p+5f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.6bee860000000p+3f, 0x1.0594c80000000p+7f, -0x1.e8a6b00000000p+8f, 0x1.a01b820000000p+9f, -0x1.4c631e0000000p+9f, 0x1.9395f40000000p+7f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.7adda80000000p+2f, 0x1.fa36e20000000p+5f, -0x1.096ec40000000p+8f, 0x1.040cec0000000p+9f, -0x1.d369800000000p+8f, 0x1.36c6100000000p+7f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.4fbfaa0000000p+3f, 0x1.a56bea0000000p+6f, -0x1.9970940000000p+8f, 0x1.6e6a6c0000000p+9f, -0x1.2f26f80000000p+9f, 0x1.78195a0000000p+7f}};
    return t[i][j];
}
__host__ __device__ constexpr float VERN7_R_LO(int i, int j) {
    constexpr float t[17][8] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.ae93600000000p-24f, -0x1.988f440000000p-20f, -0x1.f2c4b60000000p-21f, 0x1.60fa700000000p-20f, 0x1.c589f80000000p-20f, -0x1.be21d80000000p-22f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.2207300000000p-24f, 0x1.c997560000000p-19f, -0x1.39a2c00000000p-24f, -0x1.f0a3e00000000p-18f, 0x1.f05c700000000p-18f, 0x1.ac1b400000000p-20f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.354baa0000000p-22f, 0x1.9b478c0000000p-19f, -0x1.4542c60000000p-17f, 0x1.839d960000000p-16f, -0x1.587ba40000000p-16f, -0x1.40a1fa0000000p-19f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.51e6700000000p-23f, -0x1.a0429e0000000p-20f, 0x1.388c4e0000000p-18f, -0x1.f50d7a0000000p-17f, -0x1.3be2fe0000000p-18f, 0x1.65fdaa0000000p-19f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.37f3420000000p-22f, -0x1.a862bc0000000p-18f, -0x1.cbddf00000000p-20f, 0x1.ad76c20000000p-15f, 0x1.3fc4ac0000000p-20f, 0x1.a38ecc0000000p-17f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.054cc20000000p-23f, 0x1.a5fe460000000p-19f, -0x1.00cb780000000p-17f, -0x1.553ece0000000p-20f, -0x1.876ba00000000p-22f, 0x1.0add480000000p-23f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.4770aa0000000p-24f, 0x1.ada7120000000p-24f, 0x1.661a340000000p-20f, 0x1.95f4b00000000p-19f, -0x1.b0a12a0000000p-18f, 0x1.37cd1a0000000p-22f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.2caf340000000p-24f, -0x1.df15440000000p-21f, 0x1.a3abe20000000p-19f, -0x1.4bf5ea0000000p-19f, 0x1.dd7c6a0000000p-18f, 0x1.b9effa0000000p-21f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.e801c80000000p-23f, -0x1.205dec0000000p-21f, -0x1.65e27c0000000p-24f, -0x1.40f6520000000p-24f, -0x1.4613900000000p-21f, 0x1.6a9a100000000p-22f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.0580ca0000000p-22f, 0x1.33dc520000000p-20f, -0x1.482b240000000p-19f, 0x1.21c7d80000000p-24f, -0x1.fbc66c0000000p-20f, -0x1.787bea0000000p-20f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.35f6640000000p-22f, -0x1.fdc9d40000000p-18f, -0x1.ccbc3a0000000p-17f, -0x1.ab1b2e0000000p-16f, 0x1.0f51ca0000000p-16f, 0x1.b38e8a0000000p-19f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.876ec60000000p-24f, 0x1.7aa7c60000000p-20f, -0x1.0372c80000000p-18f, -0x1.c087460000000p-16f, -0x1.553d500000000p-23f, 0x1.2b721c0000000p-18f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.3bb9ce0000000p-22f, 0x1.c893920000000p-22f, 0x1.1281540000000p-17f, 0x1.d5eaac0000000p-16f, -0x1.d996220000000p-17f, 0x1.463a1a0000000p-18f}};
    return t[i][j];
}
// ROSENBROCK23: c32 = 6 + sqrt(2), d = 1 / (2 + sqrt(2)) in Float64
constexpr double ROS23_C32 = 0x1.da827999fcef3p+2;  // 7.414213562373095
constexpr float ROS23_C32_HI = 0x1.da827a0000000p+2f;
constexpr float ROS23_C32_LO = -0x1.980c440000000p-24f;
constexpr double ROS23_D = 0x1.2bec333018867p-2;  // 0.2928932188134525
constexpr float ROS23_D_HI = 0x1.2bec340000000p-2f;
constexpr float ROS23_D_LO = -0x1.9fcef40000000p-27f;
}  // namespace tab
}  // namespace odegb
