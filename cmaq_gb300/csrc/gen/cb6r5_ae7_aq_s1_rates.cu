// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cb6r5_ae7_aq/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 4242f44b2527a299).  Do not edit.
#include "cb6r5_ae7_aq_mech.cuh"
#include <math.h>
namespace mech_cb6r5_ae7_aq {
// f(y) for the day reaction list (rbfeval.F:80-151).
__device__ __noinline__ void feval_s1_0(double* __restrict__ ws, int src, int dst)
{
    const double* __restrict__ yin = ws + src;
    double* __restrict__ yout = ws + dst;
    ws[1392] = (ws[1043]) * yin[144];
    ws[1393] = (ws[1044]) * yin[130];
    ws[1394] = ((ws[1045]) * yin[135]) * yin[137];
    ws[1395] = ((ws[1046]) * yin[130]) * yin[137];
    ws[1396] = ((ws[1047]) * yin[130]) * yin[144];
    ws[1397] = ((ws[1048]) * yin[130]) * yin[144];
    ws[1398] = ((ws[1049]) * yin[130]) * yin[135];
    ws[1399] = (ws[1050]) * yin[135];
    ws[1400] = (ws[1051]) * yin[135];
    ws[1401] = (ws[1052]) * yin[21];
    ws[1402] = (ws[1053]) * yin[21];
    ws[1403] = ((ws[1054]) * yin[135]) * yin[148];
    ws[1404] = ((ws[1055]) * yin[135]) * yin[147];
    ws[1405] = ((ws[1056]) * yin[148]) * yin[130];
    ws[1406] = ((ws[1057]) * yin[147]) * yin[130];
    ws[1407] = ((ws[1058]) * yin[148]) * yin[148];
    ws[1408] = ((ws[1059]) * yin[148]) * yin[148];
    ws[1409] = ((ws[1060]) * yin[148]) * yin[147];
    ws[1410] = ((ws[1061]) * yin[147]) * yin[147];
    ws[1411] = ((ws[1062]) * yin[147]) * yin[147];
    ws[1412] = (ws[1063]) * yin[108];
    ws[1413] = ((ws[1064]) * yin[108]) * yin[148];
    ws[1414] = ((ws[1065]) * yin[108]) * yin[130];
    ws[1415] = ((ws[1066]) * yin[137]) * yin[137];
    ws[1416] = ((ws[1067]) * yin[147]) * yin[137];
    ws[1417] = ((ws[1068]) * yin[144]) * yin[135];
    ws[1418] = (ws[1069]) * yin[145];
    ws[1419] = (ws[1070]) * yin[145];
    ws[1420] = ((ws[1071]) * yin[145]) * yin[137];
    ws[1421] = ((ws[1072]) * yin[145]) * yin[144];
    ws[1422] = ((ws[1073]) * yin[145]) * yin[130];
    ws[1423] = ((ws[1074]) * yin[145]) * yin[148];
    ws[1424] = ((ws[1075]) * yin[145]) * yin[147];
    ws[1425] = ((ws[1076]) * yin[145]) * yin[135];
    ws[1426] = ((ws[1077]) * yin[145]) * yin[145];
    ws[1427] = ((ws[1078]) * yin[145]) * yin[144];
    ws[1428] = (ws[1079]) * yin[40];
    ws[1429] = (ws[1080]) * yin[40];
    ws[1430] = (ws[1081]) * yin[40];
    ws[1431] = ((ws[1082]) * yin[137]) * yin[148];
    ws[1432] = ((ws[1083]) * yin[137]) * yin[144];
    ws[1433] = ((ws[1084]) * yin[77]) * yin[77];
    ws[1434] = (ws[1085]) * yin[77];
    ws[1435] = ((ws[1086]) * yin[77]) * yin[148];
    ws[1436] = ((ws[1087]) * yin[144]) * yin[148];
    ws[1437] = ((ws[1088]) * yin[131]) * yin[148];
    ws[1438] = (ws[1089]) * yin[131];
    ws[1439] = ((ws[1090]) * yin[147]) * yin[144];
    ws[1440] = (ws[1091]) * yin[53];
    ws[1441] = (ws[1092]) * yin[53];
    ws[1442] = ((ws[1093]) * yin[53]) * yin[148];
    ws[1443] = ((ws[1094]) * yin[69]) * yin[148];
    ws[1444] = ((ws[1095]) * yin[139]) * yin[137];
    ws[1445] = ((ws[1096]) * yin[139]) * yin[144];
    ws[1446] = (ws[1097]) * yin[42];
    ws[1447] = (ws[1098]) * yin[42];
    ws[1448] = ((ws[1099]) * yin[139]) * yin[147];
    ws[1449] = ((ws[1100]) * yin[139]) * yin[146];
    ws[1450] = ((ws[1101]) * yin[139]) * yin[139];
    ws[1451] = ((ws[1102]) * yin[139]) * yin[128];
    ws[1452] = ((ws[1103]) * yin[128]) * yin[137];
    ws[1453] = ((ws[1104]) * yin[128]) * yin[144];
    ws[1454] = (ws[1105]) * yin[61];
    ws[1455] = (ws[1106]) * yin[61];
    ws[1456] = ((ws[1107]) * yin[128]) * yin[147];
    ws[1457] = ((ws[1108]) * yin[128]) * yin[146];
    ws[1458] = ((ws[1109]) * yin[128]) * yin[128];
    ws[1459] = ((ws[1110]) * yin[146]) * yin[137];
    ws[1460] = ((ws[1111]) * yin[146]) * yin[147];
    ws[1461] = ((ws[1112]) * yin[146]) * yin[146];
    ws[1462] = ((ws[1113]) * yin[138]) * yin[137];
    ws[1463] = ((ws[1114]) * yin[138]) * yin[147];
    ws[1464] = ((ws[1115]) * yin[138]) * yin[139];
    ws[1465] = ((ws[1116]) * yin[138]) * yin[146];
    ws[1466] = ((ws[1117]) * yin[143]) * yin[137];
    ws[1467] = ((ws[1118]) * yin[143]) * yin[147];
    ws[1468] = ((ws[1119]) * yin[143]) * yin[139];
    ws[1469] = ((ws[1120]) * yin[143]) * yin[146];
    ws[1470] = ((ws[1121]) * yin[136]) * yin[137];
    ws[1471] = ((ws[1122]) * yin[136]) * yin[147];
    ws[1472] = ((ws[1123]) * yin[136]) * yin[139];
    ws[1473] = ((ws[1124]) * yin[136]) * yin[146];
    ws[1474] = ((ws[1125]) * yin[134]) * yin[137];
    ws[1475] = ((ws[1126]) * yin[134]) * yin[147];
    ws[1476] = ((ws[1127]) * yin[134]) * yin[139];
    ws[1477] = ((ws[1128]) * yin[134]) * yin[146];
    ws[1478] = ((ws[1129]) * yin[71]) * yin[148];
    ws[1479] = (ws[1130]) * yin[71];
    ws[1480] = ((ws[1131]) * yin[90]) * yin[148];
    ws[1481] = (ws[1132]) * yin[90];
    ws[1482] = ((ws[1133]) * yin[114]) * yin[148];
    ws[1483] = (ws[1134]) * yin[114];
    ws[1484] = ((ws[1135]) * yin[118]) * yin[148];
    ws[1485] = ((ws[1136]) * yin[122]) * yin[148];
    ws[1486] = ((ws[1137]) * yin[84]) * yin[148];
    ws[1487] = ((ws[1138]) * yin[141]) * yin[148];
    ws[1488] = (ws[1139]) * yin[141];
    ws[1489] = (ws[1140]) * yin[141];
    ws[1490] = ((ws[1141]) * yin[141]) * yin[130];
    ws[1491] = ((ws[1142]) * yin[141]) * yin[145];
    ws[1492] = ((ws[1143]) * yin[141]) * yin[147];
    ws[1493] = (ws[1144]) * yin[54];
    ws[1494] = ((ws[1145]) * yin[54]) * yin[137];
    ws[1495] = ((ws[1146]) * yin[54]) * yin[147];
    ws[1496] = ((ws[1147]) * yin[129]) * yin[130];
    ws[1497] = ((ws[1148]) * yin[129]) * yin[148];
    ws[1498] = ((ws[1149]) * yin[129]) * yin[145];
    ws[1499] = (ws[1150]) * yin[129];
    ws[1500] = ((ws[1151]) * yin[127]) * yin[130];
    ws[1501] = ((ws[1152]) * yin[127]) * yin[148];
    ws[1502] = ((ws[1153]) * yin[127]) * yin[145];
    ws[1503] = (ws[1154]) * yin[127];
    ws[1504] = ((ws[1155]) * yin[120]) * yin[148];
    ws[1505] = (ws[1156]) * yin[120];
    ws[1506] = ((ws[1157]) * yin[120]) * yin[145];
    ws[1507] = ((ws[1158]) * yin[133]) * yin[148];
    ws[1508] = (ws[1159]) * yin[133];
    ws[1509] = ((ws[1160]) * yin[133]) * yin[145];
    ws[1510] = (ws[1161]) * yin[125];
    ws[1511] = ((ws[1162]) * yin[125]) * yin[145];
    ws[1512] = ((ws[1163]) * yin[125]) * yin[148];
    ws[1513] = (ws[1164]) * yin[148];
    ws[1514] = ((ws[1165]) * yin[140]) * yin[148];
    ws[1515] = (ws[1166]) * yin[148];
    ws[1516] = ((ws[1167]) * yin[26]) * yin[148];
    ws[1517] = ((ws[1168]) * yin[85]) * yin[148];
    ws[1518] = ((ws[1169]) * yin[27]) * yin[148];
    ws[1519] = (ws[1170]) * yin[10];
    ws[1520] = (ws[1171]) * yin[106];
    ws[1521] = ((ws[1172]) * yin[106]) * yin[148];
    ws[1522] = ((ws[1173]) * yin[28]) * yin[148];
    ws[1523] = ((ws[1174]) * yin[132]) * yin[148];
    ws[1524] = (ws[1175]) * yin[30];
    ws[1525] = (ws[1176]) * yin[30];
    ws[1526] = ((ws[1177]) * yin[30]) * yin[144];
    ws[1527] = ((ws[1178]) * yin[11]) * yin[148];
    ws[1528] = ((ws[1179]) * yin[83]) * yin[130];
    ws[1529] = ((ws[1180]) * yin[83]) * yin[148];
    ws[1530] = ((ws[1181]) * yin[83]) * yin[135];
    ws[1531] = ((ws[1182]) * yin[83]) * yin[145];
    ws[1532] = ((ws[1183]) * yin[111]) * yin[130];
    ws[1533] = ((ws[1184]) * yin[111]) * yin[148];
    ws[1534] = ((ws[1185]) * yin[111]) * yin[135];
    ws[1535] = ((ws[1186]) * yin[111]) * yin[145];
    ws[1536] = ((ws[1187]) * yin[98]) * yin[130];
    ws[1537] = ((ws[1188]) * yin[98]) * yin[148];
    ws[1538] = ((ws[1189]) * yin[98]) * yin[135];
    ws[1539] = ((ws[1190]) * yin[98]) * yin[145];
    ws[1540] = ((ws[1191]) * yin[79]) * yin[148];
    ws[1541] = ((ws[1192]) * yin[79]) * yin[130];
    ws[1542] = ((ws[1193]) * yin[107]) * yin[137];
    ws[1543] = ((ws[1194]) * yin[107]) * yin[147];
    ws[1544] = ((ws[1195]) * yin[107]) * yin[139];
    ws[1545] = ((ws[1196]) * yin[107]) * yin[146];
    ws[1546] = (ws[1197]) * yin[107];
    ws[1547] = ((ws[1198]) * yin[79]) * yin[135];
    ws[1548] = ((ws[1199]) * yin[79]) * yin[145];
    ws[1549] = ((ws[1200]) * yin[121]) * yin[148];
    ws[1550] = ((ws[1201]) * yin[121]) * yin[135];
    ws[1551] = ((ws[1202]) * yin[121]) * yin[145];
    ws[1552] = (ws[1203]) * yin[121];
    ws[1553] = ((ws[1204]) * yin[52]) * yin[148];
    ws[1554] = (ws[1205]) * yin[32];
    ws[1555] = ((ws[1206]) * yin[32]) * yin[145];
    ws[1556] = ((ws[1207]) * yin[33]) * yin[148];
    ws[1557] = ((ws[1208]) * yin[103]) * yin[147];
    ws[1558] = ((ws[1209]) * yin[103]) * yin[137];
    ws[1559] = ((ws[1210]) * yin[103]) * yin[139];
    ws[1560] = ((ws[1211]) * yin[103]) * yin[146];
    ws[1561] = ((ws[1212]) * yin[51]) * yin[148];
    ws[1562] = ((ws[1213]) * yin[64]) * yin[130];
    ws[1563] = ((ws[1214]) * yin[64]) * yin[148];
    ws[1564] = ((ws[1215]) * yin[64]) * yin[135];
    ws[1565] = ((ws[1216]) * yin[64]) * yin[145];
    ws[1566] = ((ws[1217]) * yin[66]) * yin[130];
    ws[1567] = ((ws[1218]) * yin[66]) * yin[148];
    ws[1568] = ((ws[1219]) * yin[66]) * yin[135];
    ws[1569] = ((ws[1220]) * yin[66]) * yin[145];
    ws[1570] = ((ws[1221]) * yin[12]) * yin[148];
    ws[1571] = ((ws[1222]) * yin[97]) * yin[137];
    ws[1572] = ((ws[1223]) * yin[97]) * yin[139];
    ws[1573] = ((ws[1224]) * yin[97]) * yin[147];
    ws[1574] = ((ws[1225]) * yin[97]) * yin[146];
    ws[1575] = ((ws[1226]) * yin[34]) * yin[148];
    ws[1576] = ((ws[1227]) * yin[109]) * yin[137];
    ws[1577] = ((ws[1228]) * yin[109]) * yin[139];
    ws[1578] = ((ws[1229]) * yin[109]) * yin[147];
    ws[1579] = ((ws[1230]) * yin[109]) * yin[146];
    ws[1580] = ((ws[1231]) * yin[35]) * yin[148];
    ws[1581] = ((ws[1232]) * yin[36]) * yin[148];
    ws[1582] = ((ws[1233]) * yin[112]) * yin[137];
    ws[1583] = ((ws[1234]) * yin[112]) * yin[147];
    ws[1584] = ((ws[1235]) * yin[112]) * yin[139];
    ws[1585] = ((ws[1236]) * yin[112]) * yin[146];
    ws[1586] = ((ws[1237]) * yin[113]) * yin[148];
    ws[1587] = ((ws[1238]) * yin[113]) * yin[145];
    ws[1588] = ((ws[1239]) * yin[104]) * yin[144];
    ws[1589] = ((ws[1240]) * yin[104]) * yin[147];
    ws[1590] = ((ws[1241]) * yin[68]) * yin[148];
    ws[1591] = ((ws[1242]) * yin[68]) * yin[145];
    ws[1592] = (ws[1243]) * yin[68];
    ws[1593] = (ws[1244]) * yin[119];
    ws[1594] = ((ws[1245]) * yin[119]) * yin[148];
    ws[1595] = ((ws[1246]) * yin[119]) * yin[135];
    ws[1596] = ((ws[1247]) * yin[119]) * yin[145];
    ws[1597] = (ws[1248]) * yin[123];
    ws[1598] = ((ws[1249]) * yin[123]) * yin[148];
    ws[1599] = ((ws[1250]) * yin[123]) * yin[135];
    ws[1600] = ((ws[1251]) * yin[123]) * yin[145];
    ws[1601] = ((ws[1252]) * yin[55]) * yin[148];
    ws[1602] = ((ws[1253]) * yin[55]) * yin[145];
    ws[1603] = ((ws[1254]) * yin[117]) * yin[137];
    ws[1604] = ((ws[1255]) * yin[117]) * yin[144];
    ws[1605] = (ws[1256]) * yin[56];
    ws[1606] = ((ws[1257]) * yin[117]) * yin[147];
    ws[1607] = ((ws[1258]) * yin[117]) * yin[139];
    ws[1608] = ((ws[1259]) * yin[117]) * yin[146];
    ws[1609] = ((ws[1260]) * yin[56]) * yin[148];
    ws[1610] = ((ws[1261]) * yin[61]) * yin[148];
    ws[1611] = ((ws[1262]) * yin[13]) * yin[148];
    ws[1612] = (ws[1263]) * yin[29];
    ws[1613] = (ws[1264]) * yin[29];
    ws[1614] = (ws[1265]) * yin[62];
    ws[1615] = (ws[1266]) * yin[62];
    ws[1616] = ((ws[1267]) * yin[144]) * yin[148];
    ws[1617] = (ws[1268]) * yin[37];
    ws[1618] = (ws[1269]) * yin[57];
    ws[1619] = ((ws[1270]) * yin[142]) * yin[135];
    ws[1620] = ((ws[1271]) * yin[110]) * yin[110];
    ws[1621] = ((ws[1272]) * yin[110]) * yin[137];
    ws[1622] = ((ws[1273]) * yin[110]) * yin[147];
    ws[1623] = ((ws[1274]) * yin[110]) * yin[138];
    ws[1624] = ((ws[1275]) * yin[148]) * yin[101];
    ws[1625] = (ws[1276]) * yin[101];
    ws[1626] = (ws[1277]) * yin[142];
    ws[1627] = ((ws[1278]) * yin[142]) * yin[132];
    ws[1628] = ((ws[1279]) * yin[142]) * yin[28];
    ws[1629] = ((ws[1280]) * yin[142]) * yin[26];
    ws[1630] = ((ws[1281]) * yin[142]) * yin[83];
    ws[1631] = ((ws[1282]) * yin[142]) * yin[111];
    ws[1632] = ((ws[1283]) * yin[142]) * yin[98];
    ws[1633] = ((ws[1284]) * yin[142]) * yin[79];
    ws[1634] = ((ws[1285]) * yin[142]) * yin[141];
    ws[1635] = ((ws[1286]) * yin[142]) * yin[129];
    ws[1636] = ((ws[1287]) * yin[142]) * yin[127];
    ws[1637] = ((ws[1288]) * yin[142]) * yin[85];
    ws[1638] = ((ws[1289]) * yin[142]) * yin[27];
    ws[1639] = ((ws[1290]) * yin[124]) * yin[148];
    ws[1640] = ((ws[1291]) * yin[142]) * yin[34];
    ws[1641] = ((ws[1292]) * yin[142]) * yin[35];
    ws[1642] = ((ws[1293]) * yin[142]) * yin[36];
    ws[1643] = (ws[1294]) * yin[81];
    ws[1644] = ((ws[1295]) * yin[110]) * yin[144];
    ws[1645] = (ws[1296]) * yin[38];
    ws[1646] = (ws[1297]) * yin[38];
    ws[1647] = (ws[1298]) * yin[38];
    ws[1648] = (ws[1299]) * yin[38];
    ws[1649] = ((ws[1300]) * yin[92]) * yin[137];
    ws[1650] = ((ws[1301]) * yin[92]) * yin[147];
    ws[1651] = ((ws[1302]) * yin[78]) * yin[137];
    ws[1652] = ((ws[1303]) * yin[78]) * yin[147];
    ws[1653] = ((ws[1304]) * yin[67]) * yin[137];
    ws[1654] = ((ws[1305]) * yin[67]) * yin[147];
    ws[1655] = ((ws[1306]) * yin[58]) * yin[135];
    ws[1656] = ((ws[1307]) * yin[58]) * yin[148];
    ws[1657] = ((ws[1308]) * yin[58]) * yin[145];
    ws[1658] = ((ws[1309]) * yin[80]) * yin[137];
    ws[1659] = ((ws[1310]) * yin[80]) * yin[147];
    ws[1660] = ((ws[1311]) * yin[14]) * yin[148];
    ws[1661] = (ws[1312]) * yin[126];
    ws[1662] = (ws[1313]) * yin[40];
    ws[1663] = (ws[1314]) * yin[40];
    ws[1664] = (ws[1315]) * yin[60];
    ws[1665] = (ws[1316]) * yin[39];
    ws[1666] = ((ws[1317]) * yin[60]) * yin[15];
    ws[1667] = ((ws[1318]) * yin[60]) * yin[16];
    ws[1668] = ((ws[1319]) * yin[39]) * yin[17];
    ws[1669] = (ws[1320]) * yin[144];
    ws[1670] = (ws[1321]) * yin[135];
    ws[1671] = (ws[1322]) * yin[33];
    ws[1672] = ((ws[1323]) * yin[41]) * yin[18];
    ws[1673] = (ws[1324]) * yin[41];
    ws[1674] = (ws[1325]) * yin[133];
    ws[1675] = (ws[1326]) * yin[125];
    ws[1676] = ((ws[1327]) * yin[89]) * yin[137];
    ws[1677] = ((ws[1328]) * yin[89]) * yin[147];
    ws[1678] = ((ws[1329]) * yin[89]) * yin[145];
    ws[1679] = ((ws[1330]) * yin[89]) * yin[146];
    ws[1680] = ((ws[1331]) * yin[105]) * yin[142];
    ws[1681] = ((ws[1332]) * yin[105]) * yin[148];
    ws[1682] = (ws[1333]) * yin[105];
    ws[1683] = (ws[1334]) * yin[0];
    ws[1684] = (ws[1335]) * yin[2];
    ws[1685] = (ws[1336]) * yin[3];
    ws[1686] = (ws[1337]) * yin[4];
    ws[1687] = (ws[1338]) * yin[5];
    ws[1688] = (ws[1339]) * yin[6];
    ws[1689] = (ws[1340]) * yin[7];
    ws[1690] = ((ws[1341]) * yin[22]) * yin[148];
    ws[1691] = ((ws[1342]) * yin[45]) * yin[148];
    ws[1692] = ((ws[1343]) * yin[23]) * yin[148];
    ws[1693] = ((ws[1344]) * yin[46]) * yin[148];
    ws[1694] = ((ws[1345]) * yin[24]) * yin[148];
    ws[1695] = ((ws[1346]) * yin[86]) * yin[148];
    ws[1696] = ((ws[1347]) * yin[87]) * yin[148];
    ws[1697] = ((ws[1348]) * yin[88]) * yin[148];
    ws[1698] = ((ws[1349]) * yin[72]) * yin[148];
    ws[1699] = ((ws[1350]) * yin[47]) * yin[148];
    ws[1700] = ((ws[1351]) * yin[115]) * yin[148];
    ws[1701] = ((ws[1352]) * yin[116]) * yin[148];
    ws[1702] = ((ws[1353]) * yin[91]) * yin[148];
    ws[1703] = ((ws[1354]) * yin[99]) * yin[148];
    ws[1704] = ((ws[1355]) * yin[100]) * yin[148];
    ws[1705] = ((ws[1356]) * yin[73]) * yin[148];
    ws[1706] = ((ws[1357]) * yin[73]) * yin[145];
    ws[1707] = ((ws[1358]) * yin[73]) * yin[130];
    ws[1708] = (ws[1359]) * yin[73];
    ws[1709] = (ws[1360]) * yin[73];
    ws[1710] = ((ws[1361]) * yin[73]) * yin[142];
    ws[1711] = ((ws[1362]) * yin[74]) * yin[148];
    ws[1712] = ((ws[1363]) * yin[74]) * yin[145];
    ws[1713] = ((ws[1364]) * yin[74]) * yin[130];
    ws[1714] = (ws[1365]) * yin[74];
    ws[1715] = ((ws[1366]) * yin[74]) * yin[142];
    ws[1716] = ((ws[1367]) * yin[75]) * yin[148];
    ws[1717] = ((ws[1368]) * yin[75]) * yin[135];
    ws[1718] = ((ws[1369]) * yin[75]) * yin[145];
    ws[1719] = ((ws[1370]) * yin[75]) * yin[142];
    ws[1720] = ((ws[1371]) * yin[76]) * yin[148];
    ws[1721] = ((ws[1372]) * yin[76]) * yin[135];
    ws[1722] = ((ws[1373]) * yin[76]) * yin[145];
    ws[1723] = (ws[1374]) * yin[76];
    ws[1724] = ((ws[1375]) * yin[76]) * yin[142];
    ws[1725] = ((ws[1376]) * yin[93]) * yin[148];
    ws[1726] = ((ws[1377]) * yin[93]) * yin[135];
    ws[1727] = ((ws[1378]) * yin[93]) * yin[145];
    ws[1728] = (ws[1379]) * yin[93];
    ws[1729] = ((ws[1380]) * yin[93]) * yin[142];
    ws[1730] = ((ws[1381]) * yin[48]) * yin[148];
    ws[1731] = ((ws[1382]) * yin[48]) * yin[142];
    ws[1732] = ((ws[1383]) * yin[94]) * yin[135];
    ws[1733] = ((ws[1384]) * yin[94]) * yin[37];
    ws[1734] = ((ws[1385]) * yin[94]) * yin[108];
    ws[1735] = ((ws[1386]) * yin[94]) * yin[148];
    ws[1736] = ((ws[1387]) * yin[94]) * yin[142];
    ws[1737] = ((ws[1388]) * yin[63]) * yin[148];
    ws[1738] = ((ws[1389]) * yin[63]) * yin[148];
    ws[1739] = ((ws[1390]) * yin[63]) * yin[145];
    ws[1740] = ((ws[1391]) * yin[63]) * yin[142];
    {
      double a = -ws[1683];
      yout[0] = a;
    }
    {
      double a = 1.0 * ws[1683];
      yout[1] = a;
    }
    {
      double a = -ws[1684];
      yout[2] = a;
    }
    {
      double a = -ws[1685];
      yout[3] = a;
    }
    {
      double a = -ws[1686];
      yout[4] = a;
    }
    {
      double a = -ws[1687];
      yout[5] = a;
    }
    {
      double a = -ws[1688];
      yout[6] = a;
    }
    {
      double a = -ws[1689];
      yout[7] = a;
    }
    {
      double a = 1.0 * ws[1443];
      yout[8] = a;
    }
    {
      double a = 1.0 * ws[1443];
      yout[9] = a;
    }
    {
      double a = -ws[1519];
      a = fma(0.2, ws[1524], a);
      a = fma(1.0, ws[1525], a);
      yout[10] = a;
    }
    {
      double a = -ws[1527];
      yout[11] = a;
    }
    {
      double a = -ws[1570];
      yout[12] = a;
    }
    {
      double a = -ws[1611];
      yout[13] = a;
    }
    {
      double a = -ws[1660];
      yout[14] = a;
    }
    {
      double a = -ws[1666];
      yout[15] = a;
    }
    {
      double a = -ws[1667];
      yout[16] = a;
    }
    {
      double a = -ws[1668];
      yout[17] = a;
    }
    {
      double a = -ws[1672];
      yout[18] = a;
    }
    {
      double a = 1.0 * ws[1672];
      a = fma(1.0, ws[1673], a);
      yout[19] = a;
    }
    {
      double a = 1.0 * ws[1674];
      a = fma(1.0, ws[1675], a);
      yout[20] = a;
    }
    {
      double a = 1.0 * ws[1400];
      a = a - ws[1401];
      a = a - ws[1402];
      yout[21] = a;
    }
    {
      double a = -ws[1690];
      a = fma(1.0, ws[1690], a);
      yout[22] = a;
    }
    {
      double a = -ws[1692];
      a = fma(1.0, ws[1692], a);
      yout[23] = a;
    }
    {
      double a = -ws[1694];
      yout[24] = a;
    }
    {
      double a = 1.0 * ws[1694];
      yout[25] = a;
    }
    {
      double a = -ws[1516];
      a = a - ws[1629];
      yout[26] = a;
    }
    {
      double a = -ws[1518];
      a = a - ws[1638];
      yout[27] = a;
    }
    {
      double a = -ws[1522];
      a = a - ws[1628];
      yout[28] = a;
    }
    {
      double a = 1.0 * ws[1522];
      a = a - ws[1612];
      a = a - ws[1613];
      yout[29] = a;
    }
    {
      double a = -ws[1524];
      a = fma(0.02, ws[1524], a);
      a = a - ws[1525];
      a = a - ws[1526];
      a = fma(0.874, ws[1615], a);
      yout[30] = a;
    }
    {
      double a = 1.0 * ws[1540];
      a = fma(1.0, ws[1548], a);
      yout[31] = a;
    }
    {
      double a = 1.0 * ws[1546];
      a = a - ws[1554];
      a = a - ws[1555];
      yout[32] = a;
    }
    {
      double a = 0.904 * ws[1553];
      a = a - ws[1556];
      a = a - ws[1671];
      yout[33] = a;
    }
    {
      double a = -ws[1575];
      a = a - ws[1640];
      yout[34] = a;
    }
    {
      double a = -ws[1580];
      a = a - ws[1641];
      yout[35] = a;
    }
    {
      double a = -ws[1581];
      a = a - ws[1642];
      yout[36] = a;
    }
    {
      double a = -ws[1617];
      a = fma(0.3, ws[1620], a);
      a = a - ws[1733];
      a = fma(1.0, ws[1733], a);
      yout[37] = a;
    }
    {
      double a = 1.0 * ws[1644];
      a = a - ws[1645];
      a = a - ws[1646];
      a = a - ws[1647];
      a = a - ws[1648];
      yout[38] = a;
    }
    {
      double a = 1.0 * ws[1663];
      a = a - ws[1665];
      a = a - ws[1668];
      yout[39] = a;
    }
    {
      double a = 1.0 * ws[1427];
      a = a - ws[1428];
      a = a - ws[1429];
      a = a - ws[1430];
      a = a - ws[1662];
      a = a - ws[1663];
      yout[40] = a;
    }
    {
      double a = 1.0 * ws[1671];
      a = a - ws[1672];
      a = a - ws[1673];
      yout[41] = a;
    }
    {
      double a = 1.0 * ws[1445];
      a = a - ws[1446];
      a = a - ws[1447];
      yout[42] = a;
    }
    {
      double a = 0.907 * ws[1684];
      a = fma(0.925, ws[1685], a);
      a = fma(0.943, ws[1686], a);
      yout[43] = a;
    }
    {
      double a = 0.5 * ws[1687];
      a = fma(0.5, ws[1688], a);
      a = fma(1.5, ws[1689], a);
      yout[44] = a;
    }
    {
      double a = 1.25 * ws[1690];
      a = a - ws[1691];
      yout[45] = a;
    }
    {
      double a = 1.25 * ws[1692];
      a = a - ws[1693];
      yout[46] = a;
    }
    {
      double a = 0.0023 * ws[1695];
      a = a - ws[1699];
      yout[47] = a;
    }
    {
      double a = -ws[1730];
      a = a - ws[1731];
      yout[48] = a;
    }
    {
      double a = 0.5 * ws[1732];
      a = fma(0.5, ws[1735], a);
      yout[49] = a;
    }
    {
      double a = 0.25 * ws[1738];
      a = fma(0.14, ws[1740], a);
      yout[50] = a;
    }
    {
      double a = 0.1 * ws[1542];
      a = a - ws[1561];
      a = fma(0.104, ws[1561], a);
      yout[51] = a;
    }
    {
      double a = 0.88 * ws[1543];
      a = a - ws[1553];
      yout[52] = a;
    }
    {
      double a = 1.0 * ws[1439];
      a = a - ws[1440];
      a = a - ws[1441];
      a = a - ws[1442];
      yout[53] = a;
    }
    {
      double a = 1.0 * ws[1492];
      a = a - ws[1493];
      a = a - ws[1494];
      a = a - ws[1495];
      yout[54] = a;
    }
    {
      double a = 0.732 * ws[1586];
      a = a - ws[1601];
      a = a - ws[1602];
      yout[55] = a;
    }
    {
      double a = 1.0 * ws[1604];
      a = a - ws[1605];
      a = a - ws[1609];
      yout[56] = a;
    }
    {
      double a = -ws[1618];
      a = fma(1.0, ws[1622], a);
      a = fma(1.0, ws[1647], a);
      a = fma(1.0, ws[1648], a);
      yout[57] = a;
    }
    {
      double a = -ws[1655];
      a = a - ws[1656];
      a = a - ws[1657];
      yout[58] = a;
    }
    {
      double a = 1.0 * ws[1655];
      a = fma(1.0, ws[1656], a);
      a = fma(1.0, ws[1657], a);
      yout[59] = a;
    }
    {
      double a = 1.0 * ws[1662];
      a = a - ws[1664];
      a = a - ws[1666];
      a = a - ws[1667];
      yout[60] = a;
    }
    {
      double a = 1.0 * ws[1453];
      a = a - ws[1454];
      a = a - ws[1455];
      a = a - ws[1610];
      yout[61] = a;
    }
    {
      double a = 1.0 * ws[1523];
      a = a - ws[1614];
      a = a - ws[1615];
      a = fma(1.0, ws[1627], a);
      yout[62] = a;
    }
    {
      double a = -ws[1737];
      a = a - ws[1738];
      a = a - ws[1739];
      a = a - ws[1740];
      yout[63] = a;
    }
    {
      double a = -ws[1562];
      a = a - ws[1563];
      a = a - ws[1564];
      a = a - ws[1565];
      yout[64] = a;
    }
    {
      double a = 1.0 * ws[1562];
      a = fma(1.0, ws[1563], a);
      a = fma(1.0, ws[1564], a);
      a = fma(1.0, ws[1566], a);
      a = fma(1.0, ws[1567], a);
      a = fma(1.0, ws[1568], a);
      yout[65] = a;
    }
    {
      double a = -ws[1566];
      a = a - ws[1567];
      a = a - ws[1568];
      a = a - ws[1569];
      yout[66] = a;
    }
    {
      double a = 1.0 * ws[1570];
      a = a - ws[1653];
      a = a - ws[1654];
      yout[67] = a;
    }
    {
      double a = 1.0 * ws[1588];
      a = a - ws[1590];
      a = a - ws[1591];
      a = a - ws[1592];
      yout[68] = a;
    }
    {
      double a = -ws[1443];
      a = fma(1.0, ws[1737], a);
      a = fma(0.75, ws[1738], a);
      a = fma(1.0, ws[1739], a);
      a = fma(0.86, ws[1740], a);
      yout[69] = a;
    }
    {
      double a = 0.14 * ws[1650];
      a = fma(0.193, ws[1652], a);
      a = fma(0.146, ws[1654], a);
      a = fma(0.473, ws[1659], a);
      yout[70] = a;
    }
    {
      double a = 0.9 * ws[1463];
      a = a - ws[1478];
      a = a - ws[1479];
      a = fma(0.5, ws[1495], a);
      yout[71] = a;
    }
    {
      double a = 0.0026 * ws[1695];
      a = fma(0.0035, ws[1696], a);
      a = fma(0.0005, ws[1697], a);
      a = a - ws[1698];
      a = fma(0.1043, ws[1698], a);
      yout[72] = a;
    }
    {
      double a = -ws[1705];
      a = a - ws[1706];
      a = a - ws[1707];
      a = a - ws[1708];
      a = a - ws[1709];
      a = a - ws[1710];
      yout[73] = a;
    }
    {
      double a = -ws[1711];
      a = a - ws[1712];
      a = a - ws[1713];
      a = a - ws[1714];
      a = a - ws[1715];
      yout[74] = a;
    }
    {
      double a = -ws[1716];
      a = a - ws[1717];
      a = a - ws[1718];
      a = a - ws[1719];
      yout[75] = a;
    }
    {
      double a = -ws[1720];
      a = a - ws[1721];
      a = a - ws[1722];
      a = a - ws[1723];
      a = a - ws[1724];
      yout[76] = a;
    }
    {
      double a = 1.0 * ws[1431];
      a = fma(2.0, ws[1432], a);
      a = a - ws[1433];
      a = a - ws[1433];
      a = a - ws[1434];
      a = a - ws[1435];
      a = fma(1.0, ws[1592], a);
      a = fma(0.5, ws[1669], a);
      yout[77] = a;
    }
    {
      double a = 1.0 * ws[1580];
      a = fma(1.0, ws[1641], a);
      a = a - ws[1651];
      a = a - ws[1652];
      yout[78] = a;
    }
    {
      double a = -ws[1540];
      a = a - ws[1541];
      a = a - ws[1547];
      a = a - ws[1548];
      a = a - ws[1633];
      yout[79] = a;
    }
    {
      double a = 1.0 * ws[1581];
      a = fma(1.0, ws[1642], a);
      a = a - ws[1658];
      a = a - ws[1659];
      yout[80] = a;
    }
    {
      double a = -ws[1643];
      a = fma(1.0, ws[1666], a);
      a = fma(1.0, ws[1667], a);
      a = fma(1.0, ws[1668], a);
      yout[81] = a;
    }
    {
      double a = 0.051 * ws[1649];
      a = fma(0.023, ws[1651], a);
      a = fma(0.225, ws[1658], a);
      a = fma(0.052, ws[1660], a);
      yout[82] = a;
    }
    {
      double a = -ws[1528];
      a = a - ws[1529];
      a = a - ws[1530];
      a = a - ws[1531];
      a = a - ws[1630];
      yout[83] = a;
    }
    {
      double a = 0.37 * ws[1448];
      a = fma(0.37, ws[1456], a);
      a = a - ws[1486];
      a = fma(0.37, ws[1606], a);
      yout[84] = a;
    }
    {
      double a = 0.315 * ws[1465];
      a = fma(0.15, ws[1505], a);
      a = a - ws[1517];
      a = a - ws[1637];
      yout[85] = a;
    }
    {
      double a = -ws[1695];
      a = fma(0.4857, ws[1695], a);
      a = fma(0.3003, ws[1696], a);
      a = fma(0.3856, ws[1697], a);
      a = fma(0.2181, ws[1698], a);
      a = fma(0.2412, ws[1699], a);
      yout[86] = a;
    }
    {
      double a = 0.0062 * ws[1695];
      a = a - ws[1696];
      a = fma(0.2862, ws[1696], a);
      a = fma(0.095, ws[1697], a);
      a = fma(0.3063, ws[1698], a);
      a = fma(0.2089, ws[1699], a);
      yout[87] = a;
    }
    {
      double a = 0.0025 * ws[1695];
      a = fma(0.0041, ws[1696], a);
      a = a - ws[1697];
      a = fma(0.1373, ws[1697], a);
      a = fma(0.0153, ws[1698], a);
      a = fma(0.3, ws[1699], a);
      yout[88] = a;
    }
    {
      double a = 1.0 * ws[1565];
      a = a - ws[1676];
      a = a - ws[1677];
      a = a - ws[1678];
      a = a - ws[1679];
      yout[89] = a;
    }
    {
      double a = 1.0 * ws[1467];
      a = fma(1.0, ws[1471], a);
      a = fma(1.0, ws[1475], a);
      a = a - ws[1480];
      a = a - ws[1481];
      yout[90] = a;
    }
    {
      double a = 0.0123 * ws[1700];
      a = fma(0.0139, ws[1701], a);
      a = a - ws[1702];
      a = fma(0.2607, ws[1702], a);
      a = fma(0.0491, ws[1703], a);
      a = fma(0.064, ws[1704], a);
      yout[91] = a;
    }
    {
      double a = 1.0 * ws[1575];
      a = fma(1.0, ws[1640], a);
      a = a - ws[1649];
      a = a - ws[1650];
      yout[92] = a;
    }
    {
      double a = 0.58 * ws[1716];
      a = fma(0.52, ws[1717], a);
      a = fma(0.045, ws[1718], a);
      a = fma(0.58, ws[1719], a);
      a = a - ws[1725];
      a = a - ws[1726];
      a = a - ws[1727];
      a = a - ws[1728];
      a = a - ws[1729];
      yout[93] = a;
    }
    {
      double a = -ws[1732];
      a = a - ws[1733];
      a = a - ws[1734];
      a = a - ws[1735];
      a = a - ws[1736];
      a = fma(0.5, ws[1736], a);
      yout[94] = a;
    }
    {
      double a = 0.5 * ws[1732];
      a = fma(1.0, ws[1733], a);
      a = fma(1.0, ws[1734], a);
      a = fma(0.5, ws[1735], a);
      a = fma(0.5, ws[1736], a);
      yout[95] = a;
    }
    {
      double a = 0.047 * ws[1649];
      a = fma(0.06, ws[1651], a);
      a = fma(0.392, ws[1653], a);
      a = fma(0.191, ws[1658], a);
      a = fma(0.081, ws[1660], a);
      yout[96] = a;
    }
    {
      double a = 0.352 * ws[1570];
      a = a - ws[1571];
      a = a - ws[1572];
      a = a - ws[1573];
      a = a - ws[1574];
      yout[97] = a;
    }
    {
      double a = -ws[1536];
      a = a - ws[1537];
      a = a - ws[1538];
      a = a - ws[1539];
      a = fma(0.029, ws[1553], a);
      a = a - ws[1632];
      yout[98] = a;
    }
    {
      double a = 0.0019 * ws[1695];
      a = fma(0.1239, ws[1700], a);
      a = fma(0.1027, ws[1701], a);
      a = fma(0.0702, ws[1702], a);
      a = a - ws[1703];
      a = fma(0.2577, ws[1703], a);
      a = fma(0.0385, ws[1704], a);
      yout[99] = a;
    }
    {
      double a = 0.0023 * ws[1695];
      a = fma(0.1831, ws[1700], a);
      a = fma(0.2045, ws[1701], a);
      a = fma(0.1116, ws[1702], a);
      a = fma(0.0739, ws[1703], a);
      a = a - ws[1704];
      a = fma(0.2667, ws[1704], a);
      yout[100] = a;
    }
    {
      double a = -ws[1624];
      a = a - ws[1625];
      a = fma(1.0, ws[1630], a);
      a = fma(1.0, ws[1631], a);
      a = fma(0.7, ws[1632], a);
      a = fma(1.0, ws[1633], a);
      yout[101] = a;
    }
    {
      double a = 0.016 * ws[1649];
      a = fma(0.015, ws[1651], a);
      a = fma(0.034, ws[1653], a);
      a = fma(0.028, ws[1658], a);
      a = fma(0.006, ws[1660], a);
      yout[102] = a;
    }
    {
      double a = 1.0 * ws[1556];
      a = a - ws[1557];
      a = a - ws[1558];
      a = a - ws[1559];
      a = a - ws[1560];
      yout[103] = a;
    }
    {
      double a = 0.2 * ws[1586];
      a = fma(0.3, ws[1587], a);
      a = a - ws[1588];
      a = a - ws[1589];
      a = fma(0.5, ws[1590], a);
      a = fma(0.5, ws[1591], a);
      a = fma(0.5, ws[1601], a);
      a = fma(1.0, ws[1602], a);
      yout[104] = a;
    }
    {
      double a = 0.688 * ws[1676];
      a = fma(1.0, ws[1677], a);
      a = fma(0.422, ws[1678], a);
      a = fma(0.711, ws[1679], a);
      a = a - ws[1680];
      a = fma(0.37, ws[1680], a);
      a = a - ws[1681];
      a = fma(0.24, ws[1681], a);
      a = a - ws[1682];
      yout[105] = a;
    }
    {
      double a = -ws[1520];
      a = a - ws[1521];
      a = fma(0.42, ws[1524], a);
      a = fma(0.137, ws[1549], a);
      a = fma(0.17, ws[1550], a);
      a = fma(0.17, ws[1552], a);
      a = fma(0.732, ws[1613], a);
      a = fma(1.0, ws[1628], a);
      yout[106] = a;
    }
    {
      double a = 1.0 * ws[1540];
      a = a - ws[1542];
      a = a - ws[1543];
      a = a - ws[1544];
      a = a - ws[1545];
      a = a - ws[1546];
      a = fma(0.067, ws[1553], a);
      yout[107] = a;
    }
    {
      double a = 1.0 * ws[1408];
      a = fma(1.0, ws[1410], a);
      a = fma(1.0, ws[1411], a);
      a = a - ws[1412];
      a = a - ws[1413];
      a = a - ws[1414];
      a = fma(0.04, ws[1534], a);
      a = fma(0.08, ws[1538], a);
      a = a - ws[1734];
      a = fma(1.0, ws[1734], a);
      yout[108] = a;
    }
    {
      double a = 0.65 * ws[1575];
      a = a - ws[1576];
      a = a - ws[1577];
      a = a - ws[1578];
      a = a - ws[1579];
      a = fma(0.65, ws[1640], a);
      yout[109] = a;
    }
    {
      double a = 1.0 * ws[1619];
      a = a - ws[1620];
      a = a - ws[1620];
      a = a - ws[1621];
      a = a - ws[1622];
      a = a - ws[1623];
      a = a - ws[1644];
      a = fma(1.0, ws[1645], a);
      a = fma(0.55, ws[1740], a);
      yout[110] = a;
    }
    {
      double a = -ws[1532];
      a = a - ws[1533];
      a = a - ws[1534];
      a = a - ws[1535];
      a = fma(0.24, ws[1552], a);
      a = fma(0.098, ws[1561], a);
      a = a - ws[1631];
      a = fma(0.3, ws[1632], a);
      yout[111] = a;
    }
    {
      double a = 0.544 * ws[1580];
      a = fma(0.544, ws[1581], a);
      a = a - ws[1582];
      a = a - ws[1583];
      a = a - ws[1584];
      a = a - ws[1585];
      a = fma(0.544, ws[1641], a);
      a = fma(0.544, ws[1642], a);
      yout[112] = a;
    }
    {
      double a = 0.53 * ws[1570];
      a = fma(0.18, ws[1575], a);
      a = fma(0.155, ws[1580], a);
      a = fma(0.155, ws[1581], a);
      a = a - ws[1586];
      a = a - ws[1587];
      a = fma(1.0, ws[1589], a);
      a = fma(0.18, ws[1640], a);
      a = fma(0.155, ws[1641], a);
      a = fma(0.155, ws[1642], a);
      yout[113] = a;
    }
    {
      double a = 0.5 * ws[1474];
      a = a - ws[1482];
      a = a - ws[1483];
      a = fma(1.0, ws[1526], a);
      a = fma(0.5, ws[1531], a);
      a = fma(0.5, ws[1535], a);
      a = fma(0.5, ws[1539], a);
      yout[114] = a;
    }
    {
      double a = 0.2944 * ws[1695];
      a = fma(0.2239, ws[1696], a);
      a = fma(0.2051, ws[1697], a);
      a = fma(0.1893, ws[1698], a);
      a = fma(0.2028, ws[1699], a);
      a = a - ws[1700];
      a = fma(0.6664, ws[1700], a);
      a = fma(0.2858, ws[1701], a);
      a = fma(0.3303, ws[1702], a);
      a = fma(0.3444, ws[1703], a);
      a = fma(0.3886, ws[1704], a);
      yout[115] = a;
    }
    {
      double a = 0.2021 * ws[1695];
      a = fma(0.182, ws[1696], a);
      a = fma(0.1764, ws[1697], a);
      a = fma(0.1668, ws[1698], a);
      a = fma(0.0471, ws[1699], a);
      a = fma(0.0143, ws[1700], a);
      a = a - ws[1701];
      a = fma(0.3931, ws[1701], a);
      a = fma(0.2272, ws[1702], a);
      a = fma(0.2749, ws[1703], a);
      a = fma(0.2421, ws[1704], a);
      yout[116] = a;
    }
    {
      double a = 0.457 * ws[1549];
      a = fma(0.48, ws[1587], a);
      a = fma(1.0, ws[1597], a);
      a = fma(0.6, ws[1598], a);
      a = fma(1.0, ws[1600], a);
      a = a - ws[1603];
      a = a - ws[1604];
      a = fma(1.0, ws[1605], a);
      a = a - ws[1606];
      a = a - ws[1607];
      a = a - ws[1608];
      yout[117] = a;
    }
    {
      double a = -ws[1484];
      a = fma(1.0, ws[1494], a);
      a = fma(0.5, ws[1495], a);
      a = fma(0.3, ws[1527], a);
      a = fma(0.42, ws[1530], a);
      a = fma(0.09, ws[1534], a);
      a = fma(0.15, ws[1550], a);
      a = fma(0.074, ws[1557], a);
      a = fma(0.185, ws[1561], a);
      yout[118] = a;
    }
    {
      double a = 0.2 * ws[1576];
      a = fma(0.23, ws[1577], a);
      a = fma(0.23, ws[1579], a);
      a = fma(0.244, ws[1580], a);
      a = fma(0.244, ws[1581], a);
      a = fma(0.56, ws[1582], a);
      a = fma(0.65, ws[1584], a);
      a = fma(0.65, ws[1585], a);
      a = a - ws[1593];
      a = a - ws[1594];
      a = a - ws[1595];
      a = a - ws[1596];
      a = fma(0.244, ws[1641], a);
      a = fma(0.244, ws[1642], a);
      yout[119] = a;
    }
    {
      double a = -ws[1504];
      a = a - ws[1505];
      a = a - ws[1506];
      a = fma(0.011, ws[1518], a);
      a = fma(0.22, ws[1529], a);
      a = fma(0.269, ws[1549], a);
      a = fma(0.113, ws[1551], a);
      a = fma(0.128, ws[1552], a);
      a = fma(0.275, ws[1557], a);
      a = fma(0.275, ws[1558], a);
      a = fma(0.22, ws[1559], a);
      a = fma(0.275, ws[1560], a);
      a = fma(0.331, ws[1561], a);
      yout[120] = a;
    }
    {
      double a = 0.75 * ws[1541];
      a = fma(0.9, ws[1542], a);
      a = fma(0.12, ws[1543], a);
      a = fma(1.0, ws[1544], a);
      a = fma(1.0, ws[1545], a);
      a = fma(0.65, ws[1547], a);
      a = fma(0.35, ws[1548], a);
      a = a - ws[1549];
      a = a - ws[1550];
      a = a - ws[1551];
      a = a - ws[1552];
      a = fma(1.0, ws[1554], a);
      a = fma(1.0, ws[1555], a);
      a = fma(1.0, ws[1633], a);
      yout[121] = a;
    }
    {
      double a = 0.13 * ws[1448];
      a = fma(0.13, ws[1456], a);
      a = fma(0.1, ws[1464], a);
      a = fma(0.2, ws[1468], a);
      a = fma(0.2, ws[1472], a);
      a = fma(0.2, ws[1476], a);
      a = a - ws[1485];
      a = fma(0.13, ws[1534], a);
      a = fma(0.08, ws[1538], a);
      a = fma(0.2, ws[1544], a);
      a = fma(0.2, ws[1559], a);
      a = fma(0.13, ws[1606], a);
      a = fma(0.2, ws[1608], a);
      yout[122] = a;
    }
    {
      double a = 0.118 * ws[1570];
      a = fma(0.918, ws[1571], a);
      a = fma(1.0, ws[1572], a);
      a = fma(1.0, ws[1574], a);
      a = fma(0.1, ws[1575], a);
      a = fma(0.66, ws[1576], a);
      a = fma(0.77, ws[1577], a);
      a = fma(0.77, ws[1579], a);
      a = fma(0.3, ws[1582], a);
      a = fma(0.35, ws[1584], a);
      a = fma(0.35, ws[1585], a);
      a = fma(0.025, ws[1586], a);
      a = fma(1.0, ws[1592], a);
      a = fma(0.25, ws[1596], a);
      a = a - ws[1597];
      a = a - ws[1598];
      a = a - ws[1599];
      a = a - ws[1600];
      a = fma(0.1, ws[1640], a);
      yout[123] = a;
    }
    {
      double a = 1.0 * ws[1626];
      a = fma(1.0, ws[1627], a);
      a = fma(1.0, ws[1628], a);
      a = fma(1.0, ws[1629], a);
      a = fma(0.3, ws[1632], a);
      a = fma(1.0, ws[1634], a);
      a = fma(1.0, ws[1635], a);
      a = fma(1.0, ws[1636], a);
      a = fma(1.0, ws[1637], a);
      a = fma(1.0, ws[1638], a);
      a = a - ws[1639];
      a = fma(1.0, ws[1640], a);
      a = fma(1.0, ws[1641], a);
      a = fma(1.0, ws[1642], a);
      a = fma(0.45, ws[1740], a);
      yout[124] = a;
    }
    {
      double a = -ws[1510];
      a = a - ws[1511];
      a = a - ws[1512];
      a = fma(0.075, ws[1534], a);
      a = fma(0.06, ws[1538], a);
      a = fma(0.115, ws[1549], a);
      a = fma(0.531, ws[1550], a);
      a = fma(0.113, ws[1551], a);
      a = fma(0.275, ws[1557], a);
      a = fma(0.275, ws[1558], a);
      a = fma(0.22, ws[1559], a);
      a = fma(0.275, ws[1560], a);
      a = fma(0.443, ws[1576], a);
      a = fma(0.52, ws[1577], a);
      a = fma(0.52, ws[1579], a);
      a = fma(0.675, ws[1582], a);
      a = fma(0.77, ws[1584], a);
      a = fma(0.77, ws[1585], a);
      a = fma(0.24, ws[1587], a);
      a = fma(1.0, ws[1594], a);
      a = fma(1.2, ws[1595], a);
      a = fma(0.25, ws[1596], a);
      a = fma(0.24, ws[1599], a);
      a = a - ws[1675];
      yout[125] = a;
    }
    {
      double a = 0.5 * ws[1474];
      a = fma(1.0, ws[1482], a);
      a = fma(0.65, ws[1548], a);
      a = fma(0.142, ws[1551], a);
      a = fma(0.266, ws[1561], a);
      a = fma(0.53, ws[1565], a);
      a = fma(0.53, ws[1569], a);
      a = fma(0.082, ws[1571], a);
      a = fma(0.14, ws[1576], a);
      a = fma(0.14, ws[1582], a);
      a = fma(1.0, ws[1590], a);
      a = fma(1.0, ws[1591], a);
      a = fma(0.5, ws[1596], a);
      a = fma(0.5, ws[1609], a);
      a = a - ws[1661];
      yout[126] = a;
    }
    {
      double a = -ws[1500];
      a = a - ws[1501];
      a = a - ws[1502];
      a = a - ws[1503];
      a = fma(0.37, ws[1524], a);
      a = fma(0.3, ws[1532], a);
      a = fma(0.488, ws[1533], a);
      a = fma(0.27, ws[1534], a);
      a = fma(0.375, ws[1535], a);
      a = fma(0.66, ws[1536], a);
      a = fma(0.7, ws[1537], a);
      a = fma(0.442, ws[1538], a);
      a = fma(0.625, ws[1539], a);
      a = fma(0.15, ws[1547], a);
      a = fma(0.029, ws[1553], a);
      a = fma(0.078, ws[1561], a);
      a = fma(0.15, ws[1562], a);
      a = fma(0.47, ws[1563], a);
      a = fma(0.21, ws[1564], a);
      a = fma(0.47, ws[1565], a);
      a = fma(0.15, ws[1566], a);
      a = fma(0.47, ws[1567], a);
      a = fma(0.21, ws[1568], a);
      a = fma(0.47, ws[1569], a);
      a = fma(1.0, ws[1607], a);
      a = fma(0.8, ws[1608], a);
      a = fma(0.268, ws[1613], a);
      a = fma(0.126, ws[1615], a);
      a = fma(0.67, ws[1631], a);
      a = fma(0.55, ws[1632], a);
      a = a - ws[1636];
      yout[127] = a;
    }
    {
      double a = -ws[1451];
      a = a - ws[1452];
      a = a - ws[1453];
      a = fma(1.0, ws[1454], a);
      a = fma(0.6, ws[1455], a);
      a = a - ws[1456];
      a = a - ws[1457];
      a = a - ws[1458];
      a = a - ws[1458];
      a = fma(1.0, ws[1500], a);
      a = fma(1.0, ws[1501], a);
      a = fma(1.0, ws[1502], a);
      a = fma(0.5, ws[1519], a);
      a = fma(0.25, ws[1541], a);
      a = fma(0.2, ws[1547], a);
      a = fma(0.717, ws[1551], a);
      a = fma(0.39, ws[1564], a);
      a = fma(0.39, ws[1568], a);
      a = fma(0.2, ws[1603], a);
      a = fma(1.0, ws[1636], a);
      yout[128] = a;
    }
    {
      double a = 1.0 * ws[1451];
      a = fma(1.0, ws[1452], a);
      a = fma(0.4, ws[1455], a);
      a = a - ws[1496];
      a = a - ws[1497];
      a = a - ws[1498];
      a = a - ws[1499];
      a = fma(1.0, ws[1503], a);
      a = fma(0.991, ws[1516], a);
      a = fma(0.95, ws[1518], a);
      a = fma(0.5, ws[1519], a);
      a = fma(0.74, ws[1524], a);
      a = fma(0.2, ws[1532], a);
      a = fma(0.488, ws[1533], a);
      a = fma(0.295, ws[1534], a);
      a = fma(0.25, ws[1535], a);
      a = fma(1.24, ws[1536], a);
      a = fma(1.3, ws[1537], a);
      a = fma(0.732, ws[1538], a);
      a = fma(0.5, ws[1539], a);
      a = fma(0.04, ws[1550], a);
      a = fma(0.1, ws[1595], a);
      a = fma(0.02, ws[1599], a);
      a = fma(1.0, ws[1610], a);
      a = fma(0.991, ws[1629], a);
      a = fma(0.33, ws[1631], a);
      a = fma(0.45, ws[1632], a);
      a = a - ws[1635];
      a = fma(1.0, ws[1638], a);
      yout[129] = a;
    }
    {
      double a = 1.0 * ws[1392];
      a = a - ws[1393];
      a = a - ws[1395];
      a = a - ws[1396];
      a = a - ws[1397];
      a = a - ws[1398];
      a = fma(1.0, ws[1399], a);
      a = fma(1.0, ws[1401], a);
      a = a - ws[1405];
      a = a - ws[1406];
      a = fma(1.0, ws[1407], a);
      a = a - ws[1414];
      a = fma(1.0, ws[1418], a);
      a = a - ws[1422];
      a = a - ws[1490];
      a = a - ws[1496];
      a = a - ws[1500];
      a = a - ws[1528];
      a = a - ws[1532];
      a = a - ws[1536];
      a = a - ws[1541];
      a = a - ws[1562];
      a = a - ws[1566];
      a = a - ws[1707];
      a = fma(1.0, ws[1707], a);
      a = a - ws[1713];
      a = fma(1.0, ws[1713], a);
      yout[130] = a;
    }
    {
      double a = 2.0 * ws[1430];
      a = fma(1.0, ws[1436], a);
      a = a - ws[1437];
      a = a - ws[1438];
      a = fma(1.0, ws[1491], a);
      a = fma(1.0, ws[1498], a);
      a = fma(1.0, ws[1502], a);
      a = fma(1.0, ws[1506], a);
      a = fma(1.0, ws[1509], a);
      a = fma(1.0, ws[1511], a);
      a = fma(0.717, ws[1551], a);
      a = fma(1.0, ws[1555], a);
      a = fma(1.0, ws[1587], a);
      a = fma(1.0, ws[1591], a);
      a = fma(1.0, ws[1600], a);
      a = fma(1.0, ws[1602], a);
      a = fma(1.0, ws[1616], a);
      a = fma(1.0, ws[1647], a);
      a = fma(1.0, ws[1648], a);
      a = fma(1.0, ws[1661], a);
      a = fma(1.0, ws[1662], a);
      a = fma(1.0, ws[1663], a);
      a = fma(1.0, ws[1664], a);
      a = fma(1.0, ws[1665], a);
      a = fma(0.5, ws[1669], a);
      a = fma(1.0, ws[1739], a);
      yout[131] = a;
    }
    {
      double a = -2.5 * ws[1519];
      a = a - ws[1523];
      a = fma(-2.7, ws[1524], a);
      a = fma(0.2, ws[1532], a);
      a = fma(-0.73, ws[1533], a);
      a = fma(-0.79, ws[1534], a);
      a = fma(-1.0, ws[1535], a);
      a = fma(0.1, ws[1536], a);
      a = fma(0.29, ws[1538], a);
      a = fma(1.0, ws[1539], a);
      a = fma(0.25, ws[1541], a);
      a = fma(0.35, ws[1547], a);
      a = fma(0.117, ws[1549], a);
      a = fma(0.717, ws[1551], a);
      a = fma(0.24, ws[1552], a);
      a = fma(2.175, ws[1557], a);
      a = fma(2.175, ws[1558], a);
      a = fma(1.74, ws[1559], a);
      a = fma(2.175, ws[1560], a);
      a = fma(2.7, ws[1561], a);
      a = fma(5.12, ws[1562], a);
      a = fma(1.66, ws[1563], a);
      a = fma(7.0, ws[1564], a);
      a = fma(5.12, ws[1566], a);
      a = fma(1.66, ws[1567], a);
      a = fma(7.0, ws[1568], a);
      a = fma(0.268, ws[1613], a);
      a = fma(-0.126, ws[1615], a);
      a = a - ws[1627];
      a = fma(-1.0, ws[1631], a);
      a = fma(0.3, ws[1632], a);
      yout[132] = a;
    }
    {
      double a = 0.2 * ws[1504];
      a = fma(0.11, ws[1505], a);
      a = a - ws[1507];
      a = a - ws[1508];
      a = a - ws[1509];
      a = fma(0.7, ws[1527], a);
      a = fma(0.075, ws[1534], a);
      a = fma(0.24, ws[1538], a);
      a = fma(0.17, ws[1550], a);
      a = fma(0.275, ws[1557], a);
      a = fma(0.275, ws[1558], a);
      a = fma(0.22, ws[1559], a);
      a = fma(0.275, ws[1560], a);
      a = fma(0.918, ws[1571], a);
      a = fma(1.0, ws[1572], a);
      a = fma(1.0, ws[1574], a);
      a = fma(0.417, ws[1576], a);
      a = fma(0.48, ws[1577], a);
      a = fma(0.48, ws[1579], a);
      a = fma(0.221, ws[1582], a);
      a = fma(0.26, ws[1584], a);
      a = fma(0.26, ws[1585], a);
      a = fma(0.025, ws[1586], a);
      a = fma(0.24, ws[1587], a);
      a = fma(0.4, ws[1593], a);
      a = fma(0.4, ws[1594], a);
      a = fma(0.4, ws[1598], a);
      a = fma(1.4, ws[1599], a);
      a = fma(0.5, ws[1603], a);
      a = fma(0.5, ws[1609], a);
      a = a - ws[1674];
      yout[133] = a;
    }
    {
      double a = -ws[1474];
      a = a - ws[1475];
      a = a - ws[1476];
      a = a - ws[1477];
      a = fma(0.06, ws[1480], a);
      a = fma(0.009, ws[1516], a);
      a = fma(0.04, ws[1524], a);
      a = fma(0.01, ws[1532], a);
      a = fma(0.024, ws[1533], a);
      a = fma(0.04, ws[1535], a);
      a = fma(0.04, ws[1539], a);
      a = fma(0.03, ws[1548], a);
      a = fma(0.022, ws[1549], a);
      a = fma(0.25, ws[1563], a);
      a = fma(0.18, ws[1564], a);
      a = fma(0.25, ws[1565], a);
      a = fma(0.25, ws[1567], a);
      a = fma(0.18, ws[1568], a);
      a = fma(0.25, ws[1569], a);
      a = fma(0.02, ws[1586], a);
      a = fma(0.1, ws[1587], a);
      a = fma(0.1, ws[1596], a);
      a = fma(1.0, ws[1612], a);
      a = fma(1.0, ws[1614], a);
      a = fma(0.03, ws[1628], a);
      a = fma(0.009, ws[1629], a);
      a = fma(0.04, ws[1633], a);
      yout[134] = a;
    }
    {
      double a = 1.0 * ws[1393];
      a = a - ws[1394];
      a = a - ws[1398];
      a = a - ws[1399];
      a = a - ws[1400];
      a = a - ws[1403];
      a = a - ws[1404];
      a = a - ws[1417];
      a = a - ws[1425];
      a = fma(0.13, ws[1448], a);
      a = fma(0.13, ws[1456], a);
      a = a - ws[1530];
      a = a - ws[1534];
      a = a - ws[1538];
      a = a - ws[1547];
      a = a - ws[1550];
      a = a - ws[1564];
      a = a - ws[1568];
      a = a - ws[1595];
      a = a - ws[1599];
      a = fma(0.13, ws[1606], a);
      a = a - ws[1619];
      a = a - ws[1655];
      a = fma(1.0, ws[1655], a);
      a = a - ws[1670];
      a = a - ws[1717];
      a = fma(1.0, ws[1717], a);
      a = a - ws[1721];
      a = fma(1.0, ws[1721], a);
      a = a - ws[1726];
      a = fma(1.0, ws[1726], a);
      a = a - ws[1732];
      a = fma(1.0, ws[1732], a);
      yout[135] = a;
    }
    {
      double a = -ws[1470];
      a = a - ws[1471];
      a = a - ws[1472];
      a = a - ws[1473];
      a = fma(0.2, ws[1507], a);
      a = fma(0.5, ws[1509], a);
      a = fma(1.0, ws[1511], a);
      a = fma(1.0, ws[1521], a);
      a = fma(0.5, ws[1531], a);
      a = fma(0.195, ws[1533], a);
      a = fma(0.48, ws[1535], a);
      a = fma(0.48, ws[1539], a);
      a = fma(0.25, ws[1541], a);
      a = fma(0.2, ws[1547], a);
      a = fma(0.33, ws[1548], a);
      a = fma(0.521, ws[1549], a);
      a = fma(0.142, ws[1551], a);
      a = fma(0.16, ws[1552], a);
      a = fma(0.63, ws[1561], a);
      a = fma(0.5, ws[1563], a);
      a = fma(0.69, ws[1564], a);
      a = fma(0.75, ws[1565], a);
      a = fma(0.5, ws[1567], a);
      a = fma(0.69, ws[1568], a);
      a = fma(0.75, ws[1569], a);
      a = fma(0.48, ws[1587], a);
      a = fma(0.45, ws[1596], a);
      a = fma(1.0, ws[1607], a);
      a = fma(0.874, ws[1615], a);
      a = fma(2.0, ws[1630], a);
      a = fma(2.0, ws[1631], a);
      a = fma(1.7, ws[1632], a);
      yout[136] = a;
    }
    {
      double a = 1.0 * ws[1392];
      a = a - ws[1394];
      a = a - ws[1395];
      a = fma(1.0, ws[1396], a);
      a = a - ws[1415];
      a = a - ws[1415];
      a = a - ws[1416];
      a = fma(1.0, ws[1419], a);
      a = a - ws[1420];
      a = fma(1.0, ws[1421], a);
      a = a - ws[1431];
      a = a - ws[1432];
      a = fma(1.0, ws[1433], a);
      a = fma(1.0, ws[1434], a);
      a = a - ws[1444];
      a = a - ws[1452];
      a = a - ws[1459];
      a = fma(1.0, ws[1459], a);
      a = a - ws[1462];
      a = a - ws[1466];
      a = a - ws[1470];
      a = a - ws[1474];
      a = a - ws[1494];
      a = a - ws[1542];
      a = a - ws[1558];
      a = a - ws[1571];
      a = a - ws[1576];
      a = a - ws[1582];
      a = a - ws[1603];
      a = a - ws[1621];
      a = a - ws[1649];
      a = fma(1.0, ws[1649], a);
      a = a - ws[1651];
      a = fma(1.0, ws[1651], a);
      a = a - ws[1653];
      a = fma(1.0, ws[1653], a);
      a = a - ws[1658];
      a = fma(1.0, ws[1658], a);
      a = a - ws[1676];
      a = fma(1.0, ws[1676], a);
      yout[137] = a;
    }
    {
      double a = 1.0 * ws[1444];
      a = fma(0.4, ws[1447], a);
      a = fma(0.5, ws[1448], a);
      a = fma(1.0, ws[1449], a);
      a = fma(2.0, ws[1450], a);
      a = fma(1.0, ws[1451], a);
      a = fma(0.5, ws[1456], a);
      a = fma(1.0, ws[1457], a);
      a = fma(2.0, ws[1458], a);
      a = a - ws[1462];
      a = a - ws[1463];
      a = a - ws[1464];
      a = fma(0.9, ws[1464], a);
      a = a - ws[1465];
      a = fma(0.8, ws[1468], a);
      a = fma(0.8, ws[1472], a);
      a = fma(0.8, ws[1476], a);
      a = fma(0.6, ws[1478], a);
      a = fma(1.0, ws[1479], a);
      a = fma(1.0, ws[1485], a);
      a = fma(1.0, ws[1499], a);
      a = fma(1.0, ws[1515], a);
      a = fma(0.5, ws[1519], a);
      a = fma(1.38, ws[1520], a);
      a = fma(0.8, ws[1544], a);
      a = fma(0.115, ws[1549], a);
      a = fma(0.34, ws[1552], a);
      a = fma(0.8, ws[1559], a);
      a = fma(1.0, ws[1572], a);
      a = fma(1.0, ws[1577], a);
      a = fma(1.0, ws[1584], a);
      a = fma(0.5, ws[1606], a);
      a = fma(1.0, ws[1607], a);
      a = fma(1.0, ws[1611], a);
      a = a - ws[1623];
      a = fma(1.0, ws[1626], a);
      a = fma(1.0, ws[1737], a);
      a = fma(1.0, ws[1738], a);
      a = fma(1.0, ws[1739], a);
      a = fma(1.0, ws[1740], a);
      yout[138] = a;
    }
    {
      double a = -ws[1444];
      a = a - ws[1445];
      a = fma(1.0, ws[1446], a);
      a = fma(0.6, ws[1447], a);
      a = a - ws[1448];
      a = a - ws[1449];
      a = a - ws[1450];
      a = a - ws[1450];
      a = a - ws[1451];
      a = a - ws[1464];
      a = a - ws[1468];
      a = a - ws[1472];
      a = a - ws[1476];
      a = fma(1.0, ws[1486], a);
      a = fma(1.0, ws[1496], a);
      a = fma(1.0, ws[1497], a);
      a = fma(1.0, ws[1498], a);
      a = fma(0.8, ws[1504], a);
      a = fma(1.0, ws[1506], a);
      a = fma(1.0, ws[1510], a);
      a = fma(1.0, ws[1511], a);
      a = fma(1.0, ws[1512], a);
      a = fma(0.5, ws[1519], a);
      a = fma(0.62, ws[1520], a);
      a = fma(1.0, ws[1521], a);
      a = a - ws[1544];
      a = fma(0.269, ws[1549], a);
      a = fma(0.143, ws[1550], a);
      a = fma(0.208, ws[1552], a);
      a = a - ws[1559];
      a = a - ws[1572];
      a = a - ws[1577];
      a = a - ws[1584];
      a = fma(0.3, ws[1593], a);
      a = fma(0.6, ws[1595], a);
      a = fma(0.12, ws[1599], a);
      a = a - ws[1607];
      a = fma(1.0, ws[1635], a);
      yout[139] = a;
    }
    {
      double a = 1.0 * ws[1487];
      a = fma(1.0, ws[1488], a);
      a = fma(1.0, ws[1489], a);
      a = fma(1.0, ws[1490], a);
      a = fma(1.0, ws[1491], a);
      a = fma(1.0, ws[1499], a);
      a = fma(1.0, ws[1503], a);
      a = fma(0.89, ws[1505], a);
      a = fma(1.8, ws[1507], a);
      a = fma(2.0, ws[1508], a);
      a = fma(1.5, ws[1509], a);
      a = fma(1.0, ws[1510], a);
      a = fma(1.0, ws[1512], a);
      a = a - ws[1514];
      a = fma(0.38, ws[1520], a);
      a = fma(0.3, ws[1527], a);
      a = fma(1.0, ws[1528], a);
      a = fma(0.35, ws[1530], a);
      a = fma(0.2, ws[1532], a);
      a = fma(0.378, ws[1534], a);
      a = fma(0.1, ws[1536], a);
      a = fma(0.245, ws[1538], a);
      a = fma(0.066, ws[1547], a);
      a = fma(0.137, ws[1549], a);
      a = fma(0.543, ws[1550], a);
      a = fma(0.251, ws[1557], a);
      a = fma(0.251, ws[1558], a);
      a = fma(0.2, ws[1559], a);
      a = fma(0.251, ws[1560], a);
      a = fma(0.001, ws[1564], a);
      a = fma(0.001, ws[1568], a);
      a = fma(0.7, ws[1593], a);
      a = fma(0.5, ws[1595], a);
      a = fma(1.0, ws[1597], a);
      a = fma(1.98, ws[1599], a);
      a = fma(0.5, ws[1603], a);
      a = fma(1.0, ws[1609], a);
      a = fma(1.0, ws[1624], a);
      a = fma(1.0, ws[1625], a);
      a = fma(1.0, ws[1634], a);
      yout[140] = a;
    }
    {
      double a = 1.0 * ws[1462];
      a = fma(0.1, ws[1463], a);
      a = fma(1.0, ws[1464], a);
      a = fma(0.685, ws[1465], a);
      a = fma(0.4, ws[1478], a);
      a = a - ws[1487];
      a = a - ws[1488];
      a = a - ws[1489];
      a = a - ws[1490];
      a = a - ws[1491];
      a = a - ws[1492];
      a = fma(1.0, ws[1493], a);
      a = fma(0.74, ws[1505], a);
      a = fma(1.0, ws[1517], a);
      a = fma(0.078, ws[1518], a);
      a = fma(1.0, ws[1521], a);
      a = fma(1.0, ws[1528], a);
      a = fma(1.56, ws[1529], a);
      a = fma(1.0, ws[1530], a);
      a = fma(1.125, ws[1531], a);
      a = fma(0.2, ws[1532], a);
      a = fma(0.781, ws[1533], a);
      a = fma(0.555, ws[1534], a);
      a = fma(0.5, ws[1535], a);
      a = fma(0.128, ws[1538], a);
      a = fma(0.5, ws[1541], a);
      a = fma(0.673, ws[1542], a);
      a = fma(0.12, ws[1543], a);
      a = fma(0.598, ws[1544], a);
      a = fma(0.598, ws[1545], a);
      a = fma(0.6, ws[1547], a);
      a = fma(0.35, ws[1548], a);
      a = fma(0.231, ws[1550], a);
      a = fma(0.26, ws[1552], a);
      a = fma(0.375, ws[1557], a);
      a = fma(0.375, ws[1558], a);
      a = fma(0.3, ws[1559], a);
      a = fma(0.375, ws[1560], a);
      a = fma(0.592, ws[1561], a);
      a = fma(0.28, ws[1563], a);
      a = fma(0.24, ws[1564], a);
      a = fma(0.28, ws[1567], a);
      a = fma(0.24, ws[1568], a);
      a = fma(1.0, ws[1592], a);
      a = fma(0.08, ws[1599], a);
      a = fma(0.14, ws[1601], a);
      a = fma(1.0, ws[1623], a);
      a = fma(1.0, ws[1630], a);
      a = a - ws[1634];
      a = fma(1.0, ws[1637], a);
      a = fma(1.0, ws[1737], a);
      a = fma(1.0, ws[1739], a);
      a = fma(0.45, ws[1740], a);
      yout[141] = a;
    }
    {
      double a = 2.0 * ws[1617];
      a = fma(1.0, ws[1618], a);
      a = a - ws[1619];
      a = fma(1.4, ws[1620], a);
      a = fma(1.0, ws[1621], a);
      a = fma(1.0, ws[1623], a);
      a = fma(1.0, ws[1624], a);
      a = fma(1.0, ws[1625], a);
      a = a - ws[1626];
      a = a - ws[1627];
      a = a - ws[1628];
      a = a - ws[1629];
      a = a - ws[1630];
      a = a - ws[1631];
      a = a - ws[1632];
      a = a - ws[1633];
      a = a - ws[1634];
      a = a - ws[1635];
      a = a - ws[1636];
      a = a - ws[1637];
      a = a - ws[1638];
      a = fma(1.0, ws[1639], a);
      a = a - ws[1640];
      a = a - ws[1641];
      a = a - ws[1642];
      a = fma(1.0, ws[1643], a);
      a = fma(1.0, ws[1646], a);
      a = a - ws[1680];
      a = fma(1.0, ws[1680], a);
      a = a - ws[1710];
      a = fma(1.0, ws[1710], a);
      a = a - ws[1715];
      a = fma(1.0, ws[1715], a);
      a = a - ws[1719];
      a = fma(1.0, ws[1719], a);
      a = a - ws[1724];
      a = fma(1.0, ws[1724], a);
      a = a - ws[1729];
      a = fma(1.0, ws[1729], a);
      a = a - ws[1731];
      a = fma(1.0, ws[1731], a);
      a = a - ws[1736];
      a = fma(1.0, ws[1736], a);
      a = a - ws[1740];
      yout[142] = a;
    }
    {
      double a = 1.0 * ws[1451];
      a = fma(1.0, ws[1452], a);
      a = fma(0.4, ws[1455], a);
      a = a - ws[1466];
      a = a - ws[1467];
      a = a - ws[1468];
      a = a - ws[1469];
      a = fma(0.54, ws[1480], a);
      a = fma(1.0, ws[1503], a);
      a = fma(0.11, ws[1505], a);
      a = fma(0.991, ws[1516], a);
      a = fma(0.1, ws[1518], a);
      a = fma(0.5, ws[1519], a);
      a = fma(0.94, ws[1524], a);
      a = fma(0.7, ws[1528], a);
      a = fma(1.0, ws[1529], a);
      a = fma(0.5, ws[1531], a);
      a = fma(0.2, ws[1532], a);
      a = fma(0.976, ws[1533], a);
      a = fma(0.15, ws[1534], a);
      a = fma(0.48, ws[1535], a);
      a = fma(0.1, ws[1536], a);
      a = fma(1.0, ws[1537], a);
      a = fma(0.3, ws[1538], a);
      a = fma(0.48, ws[1539], a);
      a = fma(0.082, ws[1542], a);
      a = fma(0.072, ws[1544], a);
      a = fma(0.072, ws[1545], a);
      a = fma(0.64, ws[1548], a);
      a = fma(0.142, ws[1551], a);
      a = fma(0.34, ws[1552], a);
      a = fma(0.37, ws[1561], a);
      a = fma(0.75, ws[1563], a);
      a = fma(0.07, ws[1564], a);
      a = fma(0.28, ws[1565], a);
      a = fma(0.75, ws[1567], a);
      a = fma(0.07, ws[1568], a);
      a = fma(0.28, ws[1569], a);
      a = fma(0.07, ws[1575], a);
      a = fma(0.058, ws[1580], a);
      a = fma(0.058, ws[1581], a);
      a = fma(0.12, ws[1587], a);
      a = fma(1.0, ws[1593], a);
      a = fma(2.0, ws[1594], a);
      a = fma(0.3, ws[1595], a);
      a = fma(0.45, ws[1596], a);
      a = fma(0.4, ws[1598], a);
      a = fma(0.8, ws[1608], a);
      a = fma(1.0, ws[1613], a);
      a = fma(0.126, ws[1615], a);
      a = fma(0.97, ws[1628], a);
      a = fma(0.991, ws[1629], a);
      a = fma(0.96, ws[1633], a);
      a = fma(0.07, ws[1640], a);
      a = fma(0.058, ws[1641], a);
      a = fma(0.058, ws[1642], a);
      yout[143] = a;
    }
    {
      double a = -ws[1392];
      a = fma(1.0, ws[1394], a);
      a = fma(1.0, ws[1395], a);
      a = a - ws[1396];
      a = a - ws[1397];
      a = fma(2.0, ws[1415], a);
      a = fma(1.0, ws[1416], a);
      a = a - ws[1417];
      a = fma(1.0, ws[1418], a);
      a = fma(2.0, ws[1420], a);
      a = a - ws[1421];
      a = fma(1.0, ws[1421], a);
      a = fma(1.0, ws[1422], a);
      a = fma(1.0, ws[1423], a);
      a = fma(1.0, ws[1424], a);
      a = fma(1.0, ws[1425], a);
      a = fma(2.0, ws[1426], a);
      a = a - ws[1427];
      a = fma(1.0, ws[1428], a);
      a = fma(1.0, ws[1429], a);
      a = a - ws[1432];
      a = fma(1.0, ws[1433], a);
      a = fma(1.0, ws[1435], a);
      a = a - ws[1436];
      a = fma(1.0, ws[1438], a);
      a = a - ws[1439];
      a = fma(1.0, ws[1440], a);
      a = fma(0.59, ws[1441], a);
      a = fma(1.0, ws[1442], a);
      a = fma(1.0, ws[1444], a);
      a = a - ws[1445];
      a = fma(1.0, ws[1446], a);
      a = fma(0.6, ws[1447], a);
      a = fma(1.0, ws[1452], a);
      a = a - ws[1453];
      a = fma(1.0, ws[1454], a);
      a = fma(0.6, ws[1455], a);
      a = fma(1.0, ws[1462], a);
      a = fma(1.0, ws[1466], a);
      a = fma(1.0, ws[1470], a);
      a = fma(1.0, ws[1483], a);
      a = fma(1.0, ws[1494], a);
      a = a - ws[1526];
      a = fma(0.5, ws[1531], a);
      a = fma(0.5, ws[1535], a);
      a = fma(0.5, ws[1539], a);
      a = fma(0.9, ws[1542], a);
      a = fma(0.35, ws[1548], a);
      a = fma(0.142, ws[1551], a);
      a = fma(1.0, ws[1558], a);
      a = fma(0.444, ws[1561], a);
      a = fma(0.47, ws[1565], a);
      a = fma(0.47, ws[1569], a);
      a = fma(0.918, ws[1571], a);
      a = fma(0.86, ws[1576], a);
      a = fma(0.86, ws[1582], a);
      a = a - ws[1588];
      a = fma(0.5, ws[1596], a);
      a = fma(1.0, ws[1603], a);
      a = a - ws[1604];
      a = fma(1.0, ws[1605], a);
      a = fma(0.5, ws[1609], a);
      a = fma(1.0, ws[1610], a);
      a = a - ws[1616];
      a = fma(1.0, ws[1621], a);
      a = fma(1.0, ws[1643], a);
      a = a - ws[1644];
      a = fma(1.0, ws[1645], a);
      a = a - ws[1669];
      yout[144] = a;
    }
    {
      double a = 1.0 * ws[1397];
      a = fma(1.0, ws[1417], a);
      a = a - ws[1418];
      a = a - ws[1419];
      a = a - ws[1420];
      a = a - ws[1421];
      a = a - ws[1422];
      a = a - ws[1423];
      a = a - ws[1424];
      a = a - ws[1425];
      a = a - ws[1426];
      a = a - ws[1426];
      a = a - ws[1427];
      a = fma(1.0, ws[1428], a);
      a = fma(1.0, ws[1429], a);
      a = fma(1.0, ws[1437], a);
      a = fma(0.41, ws[1441], a);
      a = fma(0.4, ws[1447], a);
      a = fma(0.4, ws[1455], a);
      a = a - ws[1491];
      a = a - ws[1498];
      a = a - ws[1502];
      a = a - ws[1506];
      a = a - ws[1509];
      a = a - ws[1511];
      a = a - ws[1531];
      a = a - ws[1535];
      a = a - ws[1539];
      a = a - ws[1548];
      a = a - ws[1551];
      a = a - ws[1555];
      a = fma(0.185, ws[1561], a);
      a = a - ws[1565];
      a = a - ws[1569];
      a = a - ws[1587];
      a = a - ws[1591];
      a = a - ws[1596];
      a = a - ws[1600];
      a = a - ws[1602];
      a = fma(1.0, ws[1646], a);
      a = a - ws[1657];
      a = fma(1.0, ws[1657], a);
      a = a - ws[1678];
      a = fma(1.0, ws[1678], a);
      a = a - ws[1706];
      a = fma(1.0, ws[1706], a);
      a = a - ws[1712];
      a = fma(1.0, ws[1712], a);
      a = a - ws[1718];
      a = fma(1.0, ws[1718], a);
      a = a - ws[1722];
      a = fma(1.0, ws[1722], a);
      a = a - ws[1727];
      a = fma(1.0, ws[1727], a);
      a = a - ws[1739];
      yout[145] = a;
    }
    {
      double a = 1.0 * ws[1444];
      a = fma(0.4, ws[1447], a);
      a = fma(0.5, ws[1448], a);
      a = a - ws[1449];
      a = fma(2.0, ws[1450], a);
      a = fma(2.0, ws[1451], a);
      a = fma(1.0, ws[1452], a);
      a = fma(0.4, ws[1455], a);
      a = fma(0.5, ws[1456], a);
      a = a - ws[1457];
      a = fma(2.0, ws[1458], a);
      a = a - ws[1459];
      a = a - ws[1460];
      a = a - ws[1461];
      a = a - ws[1461];
      a = fma(0.9, ws[1464], a);
      a = a - ws[1465];
      a = fma(1.0, ws[1465], a);
      a = fma(0.8, ws[1468], a);
      a = a - ws[1469];
      a = fma(1.0, ws[1469], a);
      a = fma(0.8, ws[1472], a);
      a = a - ws[1473];
      a = fma(1.0, ws[1473], a);
      a = fma(0.8, ws[1476], a);
      a = a - ws[1477];
      a = fma(1.0, ws[1477], a);
      a = fma(0.6, ws[1478], a);
      a = fma(1.0, ws[1479], a);
      a = fma(0.6, ws[1480], a);
      a = fma(1.0, ws[1485], a);
      a = fma(1.0, ws[1499], a);
      a = fma(1.0, ws[1503], a);
      a = fma(0.11, ws[1505], a);
      a = fma(0.2, ws[1507], a);
      a = fma(0.5, ws[1509], a);
      a = fma(1.0, ws[1511], a);
      a = fma(1.0, ws[1515], a);
      a = fma(1.0, ws[1516], a);
      a = fma(0.1, ws[1518], a);
      a = fma(1.0, ws[1519], a);
      a = fma(1.38, ws[1520], a);
      a = fma(1.0, ws[1521], a);
      a = fma(0.98, ws[1524], a);
      a = fma(0.7, ws[1528], a);
      a = fma(1.0, ws[1529], a);
      a = fma(1.0, ws[1531], a);
      a = fma(0.21, ws[1532], a);
      a = fma(1.195, ws[1533], a);
      a = fma(0.15, ws[1534], a);
      a = fma(1.0, ws[1535], a);
      a = fma(0.1, ws[1536], a);
      a = fma(1.0, ws[1537], a);
      a = fma(0.3, ws[1538], a);
      a = fma(1.0, ws[1539], a);
      a = fma(1.0, ws[1540], a);
      a = fma(0.25, ws[1541], a);
      a = fma(0.082, ws[1542], a);
      a = fma(0.872, ws[1544], a);
      a = a - ws[1545];
      a = fma(1.072, ws[1545], a);
      a = fma(0.2, ws[1547], a);
      a = fma(1.0, ws[1548], a);
      a = fma(0.658, ws[1549], a);
      a = fma(0.284, ws[1551], a);
      a = fma(0.84, ws[1552], a);
      a = fma(0.067, ws[1553], a);
      a = fma(1.0, ws[1556], a);
      a = fma(0.8, ws[1559], a);
      a = a - ws[1560];
      a = fma(1.0, ws[1560], a);
      a = fma(1.0, ws[1561], a);
      a = fma(1.5, ws[1563], a);
      a = fma(0.94, ws[1564], a);
      a = fma(1.28, ws[1565], a);
      a = fma(1.5, ws[1567], a);
      a = fma(0.94, ws[1568], a);
      a = fma(1.28, ws[1569], a);
      a = fma(0.352, ws[1570], a);
      a = fma(1.0, ws[1572], a);
      a = a - ws[1574];
      a = fma(1.0, ws[1574], a);
      a = fma(0.72, ws[1575], a);
      a = fma(1.0, ws[1577], a);
      a = a - ws[1579];
      a = fma(1.0, ws[1579], a);
      a = fma(0.602, ws[1580], a);
      a = fma(0.602, ws[1581], a);
      a = fma(1.0, ws[1584], a);
      a = a - ws[1585];
      a = fma(1.0, ws[1585], a);
      a = fma(0.02, ws[1586], a);
      a = fma(0.7, ws[1587], a);
      a = fma(2.0, ws[1594], a);
      a = fma(0.3, ws[1595], a);
      a = fma(1.0, ws[1596], a);
      a = fma(0.4, ws[1598], a);
      a = fma(0.5, ws[1606], a);
      a = fma(2.0, ws[1607], a);
      a = a - ws[1608];
      a = fma(1.8, ws[1608], a);
      a = fma(1.0, ws[1611], a);
      a = fma(1.0, ws[1612], a);
      a = fma(1.0, ws[1613], a);
      a = fma(1.0, ws[1614], a);
      a = fma(1.0, ws[1615], a);
      a = fma(1.0, ws[1626], a);
      a = fma(1.0, ws[1628], a);
      a = fma(1.0, ws[1629], a);
      a = fma(1.0, ws[1633], a);
      a = fma(0.72, ws[1640], a);
      a = fma(0.602, ws[1641], a);
      a = fma(0.602, ws[1642], a);
      a = a - ws[1679];
      a = fma(1.0, ws[1679], a);
      yout[146] = a;
    }
    {
      double a = 1.0 * ws[1403];
      a = a - ws[1404];
      a = fma(1.0, ws[1405], a);
      a = a - ws[1406];
      a = a - ws[1409];
      a = a - ws[1410];
      a = a - ws[1410];
      a = a - ws[1411];
      a = a - ws[1411];
      a = fma(1.0, ws[1413], a);
      a = fma(1.0, ws[1414], a);
      a = a - ws[1416];
      a = fma(1.0, ws[1423], a);
      a = a - ws[1424];
      a = a - ws[1439];
      a = fma(1.0, ws[1440], a);
      a = fma(0.59, ws[1441], a);
      a = fma(1.0, ws[1443], a);
      a = a - ws[1448];
      a = a - ws[1456];
      a = a - ws[1460];
      a = fma(1.0, ws[1460], a);
      a = fma(1.0, ws[1462], a);
      a = a - ws[1463];
      a = fma(0.9, ws[1464], a);
      a = fma(0.37, ws[1465], a);
      a = fma(1.0, ws[1466], a);
      a = a - ws[1467];
      a = fma(0.8, ws[1468], a);
      a = fma(0.6, ws[1469], a);
      a = a - ws[1471];
      a = a - ws[1475];
      a = fma(0.8, ws[1476], a);
      a = fma(1.0, ws[1481], a);
      a = fma(1.0, ws[1484], a);
      a = fma(1.0, ws[1487], a);
      a = fma(2.0, ws[1488], a);
      a = fma(1.0, ws[1490], a);
      a = fma(1.0, ws[1491], a);
      a = a - ws[1492];
      a = fma(1.0, ws[1493], a);
      a = fma(1.0, ws[1494], a);
      a = a - ws[1495];
      a = fma(0.2, ws[1495], a);
      a = fma(1.0, ws[1499], a);
      a = fma(1.0, ws[1503], a);
      a = fma(0.2, ws[1504], a);
      a = fma(1.4, ws[1505], a);
      a = fma(1.0, ws[1507], a);
      a = fma(2.0, ws[1508], a);
      a = fma(1.0, ws[1509], a);
      a = fma(1.0, ws[1510], a);
      a = fma(1.0, ws[1513], a);
      a = fma(1.0, ws[1514], a);
      a = fma(1.0, ws[1517], a);
      a = fma(0.9, ws[1518], a);
      a = fma(1.0, ws[1525], a);
      a = fma(0.3, ws[1527], a);
      a = fma(1.0, ws[1528], a);
      a = fma(0.27, ws[1530], a);
      a = fma(0.1, ws[1532], a);
      a = fma(0.08, ws[1534], a);
      a = fma(0.25, ws[1541], a);
      a = fma(0.818, ws[1542], a);
      a = a - ws[1543];
      a = fma(0.12, ws[1543], a);
      a = fma(0.728, ws[1544], a);
      a = fma(0.728, ws[1545], a);
      a = fma(1.0, ws[1546], a);
      a = fma(0.066, ws[1547], a);
      a = fma(0.137, ws[1549], a);
      a = fma(0.398, ws[1550], a);
      a = fma(0.76, ws[1552], a);
      a = a - ws[1557];
      a = fma(0.825, ws[1557], a);
      a = fma(0.825, ws[1558], a);
      a = fma(0.66, ws[1559], a);
      a = fma(0.825, ws[1560], a);
      a = fma(0.53, ws[1570], a);
      a = fma(0.918, ws[1571], a);
      a = fma(1.0, ws[1572], a);
      a = a - ws[1573];
      a = fma(1.0, ws[1574], a);
      a = fma(0.18, ws[1575], a);
      a = fma(0.86, ws[1576], a);
      a = fma(1.0, ws[1577], a);
      a = a - ws[1578];
      a = fma(1.0, ws[1579], a);
      a = fma(0.155, ws[1580], a);
      a = fma(0.155, ws[1581], a);
      a = fma(0.86, ws[1582], a);
      a = a - ws[1583];
      a = fma(1.0, ws[1584], a);
      a = fma(1.0, ws[1585], a);
      a = fma(1.0, ws[1586], a);
      a = a - ws[1589];
      a = fma(1.0, ws[1592], a);
      a = fma(0.7, ws[1593], a);
      a = fma(1.0, ws[1597], a);
      a = fma(0.56, ws[1599], a);
      a = fma(0.2, ws[1601], a);
      a = fma(0.8, ws[1603], a);
      a = a - ws[1606];
      a = a - ws[1622];
      a = fma(1.0, ws[1623], a);
      a = fma(1.0, ws[1625], a);
      a = fma(1.0, ws[1630], a);
      a = fma(1.0, ws[1631], a);
      a = fma(1.0, ws[1632], a);
      a = fma(1.0, ws[1634], a);
      a = fma(1.0, ws[1637], a);
      a = fma(1.0, ws[1638], a);
      a = fma(0.18, ws[1640], a);
      a = fma(0.155, ws[1641], a);
      a = fma(0.155, ws[1642], a);
      a = a - ws[1650];
      a = fma(1.0, ws[1650], a);
      a = a - ws[1652];
      a = fma(1.0, ws[1652], a);
      a = a - ws[1654];
      a = fma(1.0, ws[1654], a);
      a = a - ws[1659];
      a = fma(1.0, ws[1659], a);
      a = a - ws[1677];
      a = fma(1.0, ws[1677], a);
      yout[147] = a;
    }
    {
      double a = 2.0 * ws[1402];
      a = a - ws[1403];
      a = fma(1.0, ws[1404], a);
      a = a - ws[1405];
      a = fma(1.0, ws[1406], a);
      a = a - ws[1407];
      a = a - ws[1407];
      a = a - ws[1408];
      a = a - ws[1408];
      a = a - ws[1409];
      a = fma(2.0, ws[1412], a);
      a = a - ws[1413];
      a = fma(1.0, ws[1414], a);
      a = fma(1.0, ws[1416], a);
      a = a - ws[1423];
      a = fma(1.0, ws[1424], a);
      a = a - ws[1431];
      a = fma(1.0, ws[1434], a);
      a = a - ws[1435];
      a = a - ws[1436];
      a = a - ws[1437];
      a = fma(1.0, ws[1438], a);
      a = fma(0.41, ws[1441], a);
      a = a - ws[1442];
      a = a - ws[1443];
      a = fma(0.5, ws[1448], a);
      a = fma(0.5, ws[1456], a);
      a = a - ws[1478];
      a = fma(0.4, ws[1478], a);
      a = fma(1.0, ws[1479], a);
      a = a - ws[1480];
      a = fma(0.4, ws[1480], a);
      a = fma(1.0, ws[1481], a);
      a = a - ws[1482];
      a = a - ws[1484];
      a = a - ws[1485];
      a = a - ws[1486];
      a = a - ws[1487];
      a = fma(1.0, ws[1490], a);
      a = fma(0.2, ws[1495], a);
      a = fma(1.0, ws[1496], a);
      a = a - ws[1497];
      a = fma(1.0, ws[1500], a);
      a = a - ws[1501];
      a = a - ws[1504];
      a = fma(0.19, ws[1505], a);
      a = a - ws[1507];
      a = a - ws[1512];
      a = a - ws[1513];
      a = a - ws[1514];
      a = a - ws[1515];
      a = a - ws[1516];
      a = a - ws[1517];
      a = a - ws[1518];
      a = a - ws[1521];
      a = a - ws[1522];
      a = a - ws[1523];
      a = a - ws[1527];
      a = fma(0.7, ws[1527], a);
      a = fma(0.3, ws[1528], a);
      a = a - ws[1529];
      a = fma(0.17, ws[1530], a);
      a = fma(0.1, ws[1532], a);
      a = a - ws[1533];
      a = fma(0.334, ws[1534], a);
      a = a - ws[1537];
      a = fma(0.5, ws[1538], a);
      a = a - ws[1540];
      a = fma(0.12, ws[1543], a);
      a = fma(0.266, ws[1547], a);
      a = a - ws[1549];
      a = fma(0.461, ws[1550], a);
      a = a - ws[1553];
      a = fma(0.933, ws[1553], a);
      a = fma(1.0, ws[1554], a);
      a = a - ws[1556];
      a = fma(1.125, ws[1557], a);
      a = fma(0.125, ws[1558], a);
      a = fma(0.1, ws[1559], a);
      a = fma(0.125, ws[1560], a);
      a = a - ws[1561];
      a = a - ws[1563];
      a = fma(0.57, ws[1564], a);
      a = a - ws[1567];
      a = fma(0.57, ws[1568], a);
      a = a - ws[1570];
      a = fma(0.118, ws[1570], a);
      a = a - ws[1575];
      a = fma(0.1, ws[1575], a);
      a = a - ws[1580];
      a = fma(0.244, ws[1580], a);
      a = a - ws[1581];
      a = fma(0.244, ws[1581], a);
      a = a - ws[1586];
      a = a - ws[1590];
      a = a - ws[1594];
      a = fma(0.5, ws[1595], a);
      a = a - ws[1598];
      a = fma(0.5, ws[1599], a);
      a = a - ws[1601];
      a = fma(0.5, ws[1606], a);
      a = a - ws[1609];
      a = a - ws[1610];
      a = a - ws[1611];
      a = a - ws[1616];
      a = fma(1.0, ws[1618], a);
      a = a - ws[1624];
      a = a - ws[1639];
      a = fma(0.1, ws[1640], a);
      a = fma(0.244, ws[1641], a);
      a = fma(0.244, ws[1642], a);
      a = a - ws[1656];
      a = fma(1.0, ws[1656], a);
      a = a - ws[1660];
      a = fma(1.0, ws[1660], a);
      a = a - ws[1681];
      a = fma(1.0, ws[1681], a);
      a = a - ws[1690];
      a = fma(1.0, ws[1690], a);
      a = a - ws[1691];
      a = fma(1.0, ws[1691], a);
      a = a - ws[1692];
      a = fma(1.0, ws[1692], a);
      a = a - ws[1693];
      a = fma(1.0, ws[1693], a);
      a = a - ws[1694];
      a = fma(1.0, ws[1694], a);
      a = a - ws[1695];
      a = fma(1.0, ws[1695], a);
      a = a - ws[1696];
      a = fma(1.0, ws[1696], a);
      a = a - ws[1697];
      a = fma(1.0, ws[1697], a);
      a = a - ws[1698];
      a = fma(1.0, ws[1698], a);
      a = a - ws[1699];
      a = fma(1.0, ws[1699], a);
      a = a - ws[1700];
      a = fma(1.0, ws[1700], a);
      a = a - ws[1701];
      a = fma(1.0, ws[1701], a);
      a = a - ws[1702];
      a = fma(1.0, ws[1702], a);
      a = a - ws[1703];
      a = fma(1.0, ws[1703], a);
      a = a - ws[1704];
      a = fma(1.0, ws[1704], a);
      a = a - ws[1705];
      a = fma(1.0, ws[1705], a);
      a = a - ws[1711];
      a = fma(1.0, ws[1711], a);
      a = a - ws[1716];
      a = fma(1.0, ws[1716], a);
      a = a - ws[1720];
      a = fma(1.0, ws[1720], a);
      a = a - ws[1725];
      a = fma(1.0, ws[1725], a);
      a = a - ws[1730];
      a = fma(1.0, ws[1730], a);
      a = a - ws[1735];
      a = fma(1.0, ws[1735], a);
      a = a - ws[1737];
      a = a - ws[1738];
      yout[148] = a;
    }
}
// Partial-derivative products of 2- and 3-reactant reactions (grpderiv.F:163-189).
__device__ __noinline__ void gear_explic_s1_0(double* __restrict__ ws)
{
    const double* __restrict__ y = ws + 0;
#define CEFF_(v) ((v) <= 1.0e-30 ? 0.0 : (v))
    { const double kk = ws[1045]; ws[1741] = kk * CEFF_(y[137]); ws[1742] = kk * CEFF_(y[135]); }
    { const double kk = ws[1046]; ws[1743] = kk * CEFF_(y[137]); ws[1744] = kk * CEFF_(y[130]); }
    { const double kk = ws[1047]; ws[1745] = kk * CEFF_(y[144]); ws[1746] = kk * CEFF_(y[130]); }
    { const double kk = ws[1048]; ws[1747] = kk * CEFF_(y[144]); ws[1748] = kk * CEFF_(y[130]); }
    { const double kk = ws[1049]; ws[1749] = kk * CEFF_(y[135]); ws[1750] = kk * CEFF_(y[130]); }
    { const double kk = ws[1054]; ws[1751] = kk * CEFF_(y[148]); ws[1752] = kk * CEFF_(y[135]); }
    { const double kk = ws[1055]; ws[1753] = kk * CEFF_(y[147]); ws[1754] = kk * CEFF_(y[135]); }
    { const double kk = ws[1056]; ws[1755] = kk * CEFF_(y[130]); ws[1756] = kk * CEFF_(y[148]); }
    { const double kk = ws[1057]; ws[1757] = kk * CEFF_(y[130]); ws[1758] = kk * CEFF_(y[147]); }
    { const double kk = ws[1058]; ws[1759] = kk * CEFF_(y[148]); ws[1760] = kk * CEFF_(y[148]); }
    { const double kk = ws[1059]; ws[1761] = kk * CEFF_(y[148]); ws[1762] = kk * CEFF_(y[148]); }
    { const double kk = ws[1060]; ws[1763] = kk * CEFF_(y[147]); ws[1764] = kk * CEFF_(y[148]); }
    { const double kk = ws[1061]; ws[1765] = kk * CEFF_(y[147]); ws[1766] = kk * CEFF_(y[147]); }
    { const double kk = ws[1062]; ws[1767] = kk * CEFF_(y[147]); ws[1768] = kk * CEFF_(y[147]); }
    { const double kk = ws[1064]; ws[1769] = kk * CEFF_(y[148]); ws[1770] = kk * CEFF_(y[108]); }
    { const double kk = ws[1065]; ws[1771] = kk * CEFF_(y[130]); ws[1772] = kk * CEFF_(y[108]); }
    { const double kk = ws[1066]; ws[1773] = kk * CEFF_(y[137]); ws[1774] = kk * CEFF_(y[137]); }
    { const double kk = ws[1067]; ws[1775] = kk * CEFF_(y[137]); ws[1776] = kk * CEFF_(y[147]); }
    { const double kk = ws[1068]; ws[1777] = kk * CEFF_(y[135]); ws[1778] = kk * CEFF_(y[144]); }
    { const double kk = ws[1071]; ws[1779] = kk * CEFF_(y[137]); ws[1780] = kk * CEFF_(y[145]); }
    { const double kk = ws[1072]; ws[1781] = kk * CEFF_(y[144]); ws[1782] = kk * CEFF_(y[145]); }
    { const double kk = ws[1073]; ws[1783] = kk * CEFF_(y[130]); ws[1784] = kk * CEFF_(y[145]); }
    { const double kk = ws[1074]; ws[1785] = kk * CEFF_(y[148]); ws[1786] = kk * CEFF_(y[145]); }
    { const double kk = ws[1075]; ws[1787] = kk * CEFF_(y[147]); ws[1788] = kk * CEFF_(y[145]); }
    { const double kk = ws[1076]; ws[1789] = kk * CEFF_(y[135]); ws[1790] = kk * CEFF_(y[145]); }
    { const double kk = ws[1077]; ws[1791] = kk * CEFF_(y[145]); ws[1792] = kk * CEFF_(y[145]); }
    { const double kk = ws[1078]; ws[1793] = kk * CEFF_(y[144]); ws[1794] = kk * CEFF_(y[145]); }
    { const double kk = ws[1082]; ws[1795] = kk * CEFF_(y[148]); ws[1796] = kk * CEFF_(y[137]); }
    { const double kk = ws[1083]; ws[1797] = kk * CEFF_(y[144]); ws[1798] = kk * CEFF_(y[137]); }
    { const double kk = ws[1084]; ws[1799] = kk * CEFF_(y[77]); ws[1800] = kk * CEFF_(y[77]); }
    { const double kk = ws[1086]; ws[1801] = kk * CEFF_(y[148]); ws[1802] = kk * CEFF_(y[77]); }
    { const double kk = ws[1087]; ws[1803] = kk * CEFF_(y[148]); ws[1804] = kk * CEFF_(y[144]); }
    { const double kk = ws[1088]; ws[1805] = kk * CEFF_(y[148]); ws[1806] = kk * CEFF_(y[131]); }
    { const double kk = ws[1090]; ws[1807] = kk * CEFF_(y[144]); ws[1808] = kk * CEFF_(y[147]); }
    { const double kk = ws[1093]; ws[1809] = kk * CEFF_(y[148]); ws[1810] = kk * CEFF_(y[53]); }
    { const double kk = ws[1094]; ws[1811] = kk * CEFF_(y[148]); ws[1812] = kk * CEFF_(y[69]); }
    { const double kk = ws[1095]; ws[1813] = kk * CEFF_(y[137]); ws[1814] = kk * CEFF_(y[139]); }
    { const double kk = ws[1096]; ws[1815] = kk * CEFF_(y[144]); ws[1816] = kk * CEFF_(y[139]); }
    { const double kk = ws[1099]; ws[1817] = kk * CEFF_(y[147]); ws[1818] = kk * CEFF_(y[139]); }
    { const double kk = ws[1100]; ws[1819] = kk * CEFF_(y[146]); ws[1820] = kk * CEFF_(y[139]); }
    { const double kk = ws[1101]; ws[1821] = kk * CEFF_(y[139]); ws[1822] = kk * CEFF_(y[139]); }
    { const double kk = ws[1102]; ws[1823] = kk * CEFF_(y[128]); ws[1824] = kk * CEFF_(y[139]); }
    { const double kk = ws[1103]; ws[1825] = kk * CEFF_(y[137]); ws[1826] = kk * CEFF_(y[128]); }
    { const double kk = ws[1104]; ws[1827] = kk * CEFF_(y[144]); ws[1828] = kk * CEFF_(y[128]); }
    { const double kk = ws[1107]; ws[1829] = kk * CEFF_(y[147]); ws[1830] = kk * CEFF_(y[128]); }
    { const double kk = ws[1108]; ws[1831] = kk * CEFF_(y[146]); ws[1832] = kk * CEFF_(y[128]); }
    { const double kk = ws[1109]; ws[1833] = kk * CEFF_(y[128]); ws[1834] = kk * CEFF_(y[128]); }
    { const double kk = ws[1110]; ws[1835] = kk * CEFF_(y[137]); ws[1836] = kk * CEFF_(y[146]); }
    { const double kk = ws[1111]; ws[1837] = kk * CEFF_(y[147]); ws[1838] = kk * CEFF_(y[146]); }
    { const double kk = ws[1112]; ws[1839] = kk * CEFF_(y[146]); ws[1840] = kk * CEFF_(y[146]); }
    { const double kk = ws[1113]; ws[1841] = kk * CEFF_(y[137]); ws[1842] = kk * CEFF_(y[138]); }
    { const double kk = ws[1114]; ws[1843] = kk * CEFF_(y[147]); ws[1844] = kk * CEFF_(y[138]); }
    { const double kk = ws[1115]; ws[1845] = kk * CEFF_(y[139]); ws[1846] = kk * CEFF_(y[138]); }
    { const double kk = ws[1116]; ws[1847] = kk * CEFF_(y[146]); ws[1848] = kk * CEFF_(y[138]); }
    { const double kk = ws[1117]; ws[1849] = kk * CEFF_(y[137]); ws[1850] = kk * CEFF_(y[143]); }
    { const double kk = ws[1118]; ws[1851] = kk * CEFF_(y[147]); ws[1852] = kk * CEFF_(y[143]); }
    { const double kk = ws[1119]; ws[1853] = kk * CEFF_(y[139]); ws[1854] = kk * CEFF_(y[143]); }
    { const double kk = ws[1120]; ws[1855] = kk * CEFF_(y[146]); ws[1856] = kk * CEFF_(y[143]); }
    { const double kk = ws[1121]; ws[1857] = kk * CEFF_(y[137]); ws[1858] = kk * CEFF_(y[136]); }
    { const double kk = ws[1122]; ws[1859] = kk * CEFF_(y[147]); ws[1860] = kk * CEFF_(y[136]); }
    { const double kk = ws[1123]; ws[1861] = kk * CEFF_(y[139]); ws[1862] = kk * CEFF_(y[136]); }
    { const double kk = ws[1124]; ws[1863] = kk * CEFF_(y[146]); ws[1864] = kk * CEFF_(y[136]); }
    { const double kk = ws[1125]; ws[1865] = kk * CEFF_(y[137]); ws[1866] = kk * CEFF_(y[134]); }
    { const double kk = ws[1126]; ws[1867] = kk * CEFF_(y[147]); ws[1868] = kk * CEFF_(y[134]); }
    { const double kk = ws[1127]; ws[1869] = kk * CEFF_(y[139]); ws[1870] = kk * CEFF_(y[134]); }
    { const double kk = ws[1128]; ws[1871] = kk * CEFF_(y[146]); ws[1872] = kk * CEFF_(y[134]); }
    { const double kk = ws[1129]; ws[1873] = kk * CEFF_(y[148]); ws[1874] = kk * CEFF_(y[71]); }
    { const double kk = ws[1131]; ws[1875] = kk * CEFF_(y[148]); ws[1876] = kk * CEFF_(y[90]); }
    { const double kk = ws[1133]; ws[1877] = kk * CEFF_(y[148]); ws[1878] = kk * CEFF_(y[114]); }
    { const double kk = ws[1135]; ws[1879] = kk * CEFF_(y[148]); ws[1880] = kk * CEFF_(y[118]); }
    { const double kk = ws[1136]; ws[1881] = kk * CEFF_(y[148]); ws[1882] = kk * CEFF_(y[122]); }
    { const double kk = ws[1137]; ws[1883] = kk * CEFF_(y[148]); ws[1884] = kk * CEFF_(y[84]); }
    { const double kk = ws[1138]; ws[1885] = kk * CEFF_(y[148]); ws[1886] = kk * CEFF_(y[141]); }
    { const double kk = ws[1141]; ws[1887] = kk * CEFF_(y[130]); ws[1888] = kk * CEFF_(y[141]); }
    { const double kk = ws[1142]; ws[1889] = kk * CEFF_(y[145]); ws[1890] = kk * CEFF_(y[141]); }
    { const double kk = ws[1143]; ws[1891] = kk * CEFF_(y[147]); ws[1892] = kk * CEFF_(y[141]); }
    { const double kk = ws[1145]; ws[1893] = kk * CEFF_(y[137]); ws[1894] = kk * CEFF_(y[54]); }
    { const double kk = ws[1146]; ws[1895] = kk * CEFF_(y[147]); ws[1896] = kk * CEFF_(y[54]); }
    { const double kk = ws[1147]; ws[1897] = kk * CEFF_(y[130]); ws[1898] = kk * CEFF_(y[129]); }
    { const double kk = ws[1148]; ws[1899] = kk * CEFF_(y[148]); ws[1900] = kk * CEFF_(y[129]); }
    { const double kk = ws[1149]; ws[1901] = kk * CEFF_(y[145]); ws[1902] = kk * CEFF_(y[129]); }
    { const double kk = ws[1151]; ws[1903] = kk * CEFF_(y[130]); ws[1904] = kk * CEFF_(y[127]); }
    { const double kk = ws[1152]; ws[1905] = kk * CEFF_(y[148]); ws[1906] = kk * CEFF_(y[127]); }
    { const double kk = ws[1153]; ws[1907] = kk * CEFF_(y[145]); ws[1908] = kk * CEFF_(y[127]); }
    { const double kk = ws[1155]; ws[1909] = kk * CEFF_(y[148]); ws[1910] = kk * CEFF_(y[120]); }
    { const double kk = ws[1157]; ws[1911] = kk * CEFF_(y[145]); ws[1912] = kk * CEFF_(y[120]); }
    { const double kk = ws[1158]; ws[1913] = kk * CEFF_(y[148]); ws[1914] = kk * CEFF_(y[133]); }
    { const double kk = ws[1160]; ws[1915] = kk * CEFF_(y[145]); ws[1916] = kk * CEFF_(y[133]); }
    { const double kk = ws[1162]; ws[1917] = kk * CEFF_(y[145]); ws[1918] = kk * CEFF_(y[125]); }
    { const double kk = ws[1163]; ws[1919] = kk * CEFF_(y[148]); ws[1920] = kk * CEFF_(y[125]); }
    { const double kk = ws[1165]; ws[1921] = kk * CEFF_(y[148]); ws[1922] = kk * CEFF_(y[140]); }
    { const double kk = ws[1167]; ws[1923] = kk * CEFF_(y[148]); ws[1924] = kk * CEFF_(y[26]); }
    { const double kk = ws[1168]; ws[1925] = kk * CEFF_(y[148]); ws[1926] = kk * CEFF_(y[85]); }
    { const double kk = ws[1169]; ws[1927] = kk * CEFF_(y[148]); ws[1928] = kk * CEFF_(y[27]); }
    { const double kk = ws[1172]; ws[1929] = kk * CEFF_(y[148]); ws[1930] = kk * CEFF_(y[106]); }
    { const double kk = ws[1173]; ws[1931] = kk * CEFF_(y[148]); ws[1932] = kk * CEFF_(y[28]); }
    { const double kk = ws[1174]; ws[1933] = kk * CEFF_(y[148]); ws[1934] = kk * CEFF_(y[132]); }
    { const double kk = ws[1177]; ws[1935] = kk * CEFF_(y[144]); ws[1936] = kk * CEFF_(y[30]); }
    { const double kk = ws[1178]; ws[1937] = kk * CEFF_(y[148]); ws[1938] = kk * CEFF_(y[11]); }
    { const double kk = ws[1179]; ws[1939] = kk * CEFF_(y[130]); ws[1940] = kk * CEFF_(y[83]); }
    { const double kk = ws[1180]; ws[1941] = kk * CEFF_(y[148]); ws[1942] = kk * CEFF_(y[83]); }
    { const double kk = ws[1181]; ws[1943] = kk * CEFF_(y[135]); ws[1944] = kk * CEFF_(y[83]); }
    { const double kk = ws[1182]; ws[1945] = kk * CEFF_(y[145]); ws[1946] = kk * CEFF_(y[83]); }
    { const double kk = ws[1183]; ws[1947] = kk * CEFF_(y[130]); ws[1948] = kk * CEFF_(y[111]); }
    { const double kk = ws[1184]; ws[1949] = kk * CEFF_(y[148]); ws[1950] = kk * CEFF_(y[111]); }
    { const double kk = ws[1185]; ws[1951] = kk * CEFF_(y[135]); ws[1952] = kk * CEFF_(y[111]); }
    { const double kk = ws[1186]; ws[1953] = kk * CEFF_(y[145]); ws[1954] = kk * CEFF_(y[111]); }
    { const double kk = ws[1187]; ws[1955] = kk * CEFF_(y[130]); ws[1956] = kk * CEFF_(y[98]); }
    { const double kk = ws[1188]; ws[1957] = kk * CEFF_(y[148]); ws[1958] = kk * CEFF_(y[98]); }
    { const double kk = ws[1189]; ws[1959] = kk * CEFF_(y[135]); ws[1960] = kk * CEFF_(y[98]); }
    { const double kk = ws[1190]; ws[1961] = kk * CEFF_(y[145]); ws[1962] = kk * CEFF_(y[98]); }
    { const double kk = ws[1191]; ws[1963] = kk * CEFF_(y[148]); ws[1964] = kk * CEFF_(y[79]); }
    { const double kk = ws[1192]; ws[1965] = kk * CEFF_(y[130]); ws[1966] = kk * CEFF_(y[79]); }
    { const double kk = ws[1193]; ws[1967] = kk * CEFF_(y[137]); ws[1968] = kk * CEFF_(y[107]); }
    { const double kk = ws[1194]; ws[1969] = kk * CEFF_(y[147]); ws[1970] = kk * CEFF_(y[107]); }
    { const double kk = ws[1195]; ws[1971] = kk * CEFF_(y[139]); ws[1972] = kk * CEFF_(y[107]); }
    { const double kk = ws[1196]; ws[1973] = kk * CEFF_(y[146]); ws[1974] = kk * CEFF_(y[107]); }
    { const double kk = ws[1198]; ws[1975] = kk * CEFF_(y[135]); ws[1976] = kk * CEFF_(y[79]); }
    { const double kk = ws[1199]; ws[1977] = kk * CEFF_(y[145]); ws[1978] = kk * CEFF_(y[79]); }
    { const double kk = ws[1200]; ws[1979] = kk * CEFF_(y[148]); ws[1980] = kk * CEFF_(y[121]); }
    { const double kk = ws[1201]; ws[1981] = kk * CEFF_(y[135]); ws[1982] = kk * CEFF_(y[121]); }
    { const double kk = ws[1202]; ws[1983] = kk * CEFF_(y[145]); ws[1984] = kk * CEFF_(y[121]); }
    { const double kk = ws[1204]; ws[1985] = kk * CEFF_(y[148]); ws[1986] = kk * CEFF_(y[52]); }
    { const double kk = ws[1206]; ws[1987] = kk * CEFF_(y[145]); ws[1988] = kk * CEFF_(y[32]); }
    { const double kk = ws[1207]; ws[1989] = kk * CEFF_(y[148]); ws[1990] = kk * CEFF_(y[33]); }
    { const double kk = ws[1208]; ws[1991] = kk * CEFF_(y[147]); ws[1992] = kk * CEFF_(y[103]); }
    { const double kk = ws[1209]; ws[1993] = kk * CEFF_(y[137]); ws[1994] = kk * CEFF_(y[103]); }
    { const double kk = ws[1210]; ws[1995] = kk * CEFF_(y[139]); ws[1996] = kk * CEFF_(y[103]); }
    { const double kk = ws[1211]; ws[1997] = kk * CEFF_(y[146]); ws[1998] = kk * CEFF_(y[103]); }
    { const double kk = ws[1212]; ws[1999] = kk * CEFF_(y[148]); ws[2000] = kk * CEFF_(y[51]); }
    { const double kk = ws[1213]; ws[2001] = kk * CEFF_(y[130]); ws[2002] = kk * CEFF_(y[64]); }
    { const double kk = ws[1214]; ws[2003] = kk * CEFF_(y[148]); ws[2004] = kk * CEFF_(y[64]); }
    { const double kk = ws[1215]; ws[2005] = kk * CEFF_(y[135]); ws[2006] = kk * CEFF_(y[64]); }
    { const double kk = ws[1216]; ws[2007] = kk * CEFF_(y[145]); ws[2008] = kk * CEFF_(y[64]); }
    { const double kk = ws[1217]; ws[2009] = kk * CEFF_(y[130]); ws[2010] = kk * CEFF_(y[66]); }
    { const double kk = ws[1218]; ws[2011] = kk * CEFF_(y[148]); ws[2012] = kk * CEFF_(y[66]); }
    { const double kk = ws[1219]; ws[2013] = kk * CEFF_(y[135]); ws[2014] = kk * CEFF_(y[66]); }
    { const double kk = ws[1220]; ws[2015] = kk * CEFF_(y[145]); ws[2016] = kk * CEFF_(y[66]); }
    { const double kk = ws[1221]; ws[2017] = kk * CEFF_(y[148]); ws[2018] = kk * CEFF_(y[12]); }
    { const double kk = ws[1222]; ws[2019] = kk * CEFF_(y[137]); ws[2020] = kk * CEFF_(y[97]); }
    { const double kk = ws[1223]; ws[2021] = kk * CEFF_(y[139]); ws[2022] = kk * CEFF_(y[97]); }
    { const double kk = ws[1224]; ws[2023] = kk * CEFF_(y[147]); ws[2024] = kk * CEFF_(y[97]); }
    { const double kk = ws[1225]; ws[2025] = kk * CEFF_(y[146]); ws[2026] = kk * CEFF_(y[97]); }
    { const double kk = ws[1226]; ws[2027] = kk * CEFF_(y[148]); ws[2028] = kk * CEFF_(y[34]); }
    { const double kk = ws[1227]; ws[2029] = kk * CEFF_(y[137]); ws[2030] = kk * CEFF_(y[109]); }
    { const double kk = ws[1228]; ws[2031] = kk * CEFF_(y[139]); ws[2032] = kk * CEFF_(y[109]); }
    { const double kk = ws[1229]; ws[2033] = kk * CEFF_(y[147]); ws[2034] = kk * CEFF_(y[109]); }
    { const double kk = ws[1230]; ws[2035] = kk * CEFF_(y[146]); ws[2036] = kk * CEFF_(y[109]); }
    { const double kk = ws[1231]; ws[2037] = kk * CEFF_(y[148]); ws[2038] = kk * CEFF_(y[35]); }
    { const double kk = ws[1232]; ws[2039] = kk * CEFF_(y[148]); ws[2040] = kk * CEFF_(y[36]); }
    { const double kk = ws[1233]; ws[2041] = kk * CEFF_(y[137]); ws[2042] = kk * CEFF_(y[112]); }
    { const double kk = ws[1234]; ws[2043] = kk * CEFF_(y[147]); ws[2044] = kk * CEFF_(y[112]); }
    { const double kk = ws[1235]; ws[2045] = kk * CEFF_(y[139]); ws[2046] = kk * CEFF_(y[112]); }
    { const double kk = ws[1236]; ws[2047] = kk * CEFF_(y[146]); ws[2048] = kk * CEFF_(y[112]); }
    { const double kk = ws[1237]; ws[2049] = kk * CEFF_(y[148]); ws[2050] = kk * CEFF_(y[113]); }
    { const double kk = ws[1238]; ws[2051] = kk * CEFF_(y[145]); ws[2052] = kk * CEFF_(y[113]); }
    { const double kk = ws[1239]; ws[2053] = kk * CEFF_(y[144]); ws[2054] = kk * CEFF_(y[104]); }
    { const double kk = ws[1240]; ws[2055] = kk * CEFF_(y[147]); ws[2056] = kk * CEFF_(y[104]); }
    { const double kk = ws[1241]; ws[2057] = kk * CEFF_(y[148]); ws[2058] = kk * CEFF_(y[68]); }
    { const double kk = ws[1242]; ws[2059] = kk * CEFF_(y[145]); ws[2060] = kk * CEFF_(y[68]); }
    { const double kk = ws[1245]; ws[2061] = kk * CEFF_(y[148]); ws[2062] = kk * CEFF_(y[119]); }
    { const double kk = ws[1246]; ws[2063] = kk * CEFF_(y[135]); ws[2064] = kk * CEFF_(y[119]); }
    { const double kk = ws[1247]; ws[2065] = kk * CEFF_(y[145]); ws[2066] = kk * CEFF_(y[119]); }
    { const double kk = ws[1249]; ws[2067] = kk * CEFF_(y[148]); ws[2068] = kk * CEFF_(y[123]); }
    { const double kk = ws[1250]; ws[2069] = kk * CEFF_(y[135]); ws[2070] = kk * CEFF_(y[123]); }
    { const double kk = ws[1251]; ws[2071] = kk * CEFF_(y[145]); ws[2072] = kk * CEFF_(y[123]); }
    { const double kk = ws[1252]; ws[2073] = kk * CEFF_(y[148]); ws[2074] = kk * CEFF_(y[55]); }
    { const double kk = ws[1253]; ws[2075] = kk * CEFF_(y[145]); ws[2076] = kk * CEFF_(y[55]); }
    { const double kk = ws[1254]; ws[2077] = kk * CEFF_(y[137]); ws[2078] = kk * CEFF_(y[117]); }
    { const double kk = ws[1255]; ws[2079] = kk * CEFF_(y[144]); ws[2080] = kk * CEFF_(y[117]); }
    { const double kk = ws[1257]; ws[2081] = kk * CEFF_(y[147]); ws[2082] = kk * CEFF_(y[117]); }
    { const double kk = ws[1258]; ws[2083] = kk * CEFF_(y[139]); ws[2084] = kk * CEFF_(y[117]); }
    { const double kk = ws[1259]; ws[2085] = kk * CEFF_(y[146]); ws[2086] = kk * CEFF_(y[117]); }
    { const double kk = ws[1260]; ws[2087] = kk * CEFF_(y[148]); ws[2088] = kk * CEFF_(y[56]); }
    { const double kk = ws[1261]; ws[2089] = kk * CEFF_(y[148]); ws[2090] = kk * CEFF_(y[61]); }
    { const double kk = ws[1262]; ws[2091] = kk * CEFF_(y[148]); ws[2092] = kk * CEFF_(y[13]); }
    { const double kk = ws[1267]; ws[2093] = kk * CEFF_(y[148]); ws[2094] = kk * CEFF_(y[144]); }
    { const double kk = ws[1270]; ws[2095] = kk * CEFF_(y[135]); ws[2096] = kk * CEFF_(y[142]); }
    { const double kk = ws[1271]; ws[2097] = kk * CEFF_(y[110]); ws[2098] = kk * CEFF_(y[110]); }
    { const double kk = ws[1272]; ws[2099] = kk * CEFF_(y[137]); ws[2100] = kk * CEFF_(y[110]); }
    { const double kk = ws[1273]; ws[2101] = kk * CEFF_(y[147]); ws[2102] = kk * CEFF_(y[110]); }
    { const double kk = ws[1274]; ws[2103] = kk * CEFF_(y[138]); ws[2104] = kk * CEFF_(y[110]); }
    { const double kk = ws[1275]; ws[2105] = kk * CEFF_(y[101]); ws[2106] = kk * CEFF_(y[148]); }
    { const double kk = ws[1278]; ws[2107] = kk * CEFF_(y[132]); ws[2108] = kk * CEFF_(y[142]); }
    { const double kk = ws[1279]; ws[2109] = kk * CEFF_(y[28]); ws[2110] = kk * CEFF_(y[142]); }
    { const double kk = ws[1280]; ws[2111] = kk * CEFF_(y[26]); ws[2112] = kk * CEFF_(y[142]); }
    { const double kk = ws[1281]; ws[2113] = kk * CEFF_(y[83]); ws[2114] = kk * CEFF_(y[142]); }
    { const double kk = ws[1282]; ws[2115] = kk * CEFF_(y[111]); ws[2116] = kk * CEFF_(y[142]); }
    { const double kk = ws[1283]; ws[2117] = kk * CEFF_(y[98]); ws[2118] = kk * CEFF_(y[142]); }
    { const double kk = ws[1284]; ws[2119] = kk * CEFF_(y[79]); ws[2120] = kk * CEFF_(y[142]); }
    { const double kk = ws[1285]; ws[2121] = kk * CEFF_(y[141]); ws[2122] = kk * CEFF_(y[142]); }
    { const double kk = ws[1286]; ws[2123] = kk * CEFF_(y[129]); ws[2124] = kk * CEFF_(y[142]); }
    { const double kk = ws[1287]; ws[2125] = kk * CEFF_(y[127]); ws[2126] = kk * CEFF_(y[142]); }
    { const double kk = ws[1288]; ws[2127] = kk * CEFF_(y[85]); ws[2128] = kk * CEFF_(y[142]); }
    { const double kk = ws[1289]; ws[2129] = kk * CEFF_(y[27]); ws[2130] = kk * CEFF_(y[142]); }
    { const double kk = ws[1290]; ws[2131] = kk * CEFF_(y[148]); ws[2132] = kk * CEFF_(y[124]); }
    { const double kk = ws[1291]; ws[2133] = kk * CEFF_(y[34]); ws[2134] = kk * CEFF_(y[142]); }
    { const double kk = ws[1292]; ws[2135] = kk * CEFF_(y[35]); ws[2136] = kk * CEFF_(y[142]); }
    { const double kk = ws[1293]; ws[2137] = kk * CEFF_(y[36]); ws[2138] = kk * CEFF_(y[142]); }
    { const double kk = ws[1295]; ws[2139] = kk * CEFF_(y[144]); ws[2140] = kk * CEFF_(y[110]); }
    { const double kk = ws[1300]; ws[2141] = kk * CEFF_(y[137]); ws[2142] = kk * CEFF_(y[92]); }
    { const double kk = ws[1301]; ws[2143] = kk * CEFF_(y[147]); ws[2144] = kk * CEFF_(y[92]); }
    { const double kk = ws[1302]; ws[2145] = kk * CEFF_(y[137]); ws[2146] = kk * CEFF_(y[78]); }
    { const double kk = ws[1303]; ws[2147] = kk * CEFF_(y[147]); ws[2148] = kk * CEFF_(y[78]); }
    { const double kk = ws[1304]; ws[2149] = kk * CEFF_(y[137]); ws[2150] = kk * CEFF_(y[67]); }
    { const double kk = ws[1305]; ws[2151] = kk * CEFF_(y[147]); ws[2152] = kk * CEFF_(y[67]); }
    { const double kk = ws[1306]; ws[2153] = kk * CEFF_(y[135]); ws[2154] = kk * CEFF_(y[58]); }
    { const double kk = ws[1307]; ws[2155] = kk * CEFF_(y[148]); ws[2156] = kk * CEFF_(y[58]); }
    { const double kk = ws[1308]; ws[2157] = kk * CEFF_(y[145]); ws[2158] = kk * CEFF_(y[58]); }
    { const double kk = ws[1309]; ws[2159] = kk * CEFF_(y[137]); ws[2160] = kk * CEFF_(y[80]); }
    { const double kk = ws[1310]; ws[2161] = kk * CEFF_(y[147]); ws[2162] = kk * CEFF_(y[80]); }
    { const double kk = ws[1311]; ws[2163] = kk * CEFF_(y[148]); ws[2164] = kk * CEFF_(y[14]); }
    { const double kk = ws[1317]; ws[2165] = kk * CEFF_(y[15]); ws[2166] = kk * CEFF_(y[60]); }
    { const double kk = ws[1318]; ws[2167] = kk * CEFF_(y[16]); ws[2168] = kk * CEFF_(y[60]); }
    { const double kk = ws[1319]; ws[2169] = kk * CEFF_(y[17]); ws[2170] = kk * CEFF_(y[39]); }
    { const double kk = ws[1323]; ws[2171] = kk * CEFF_(y[18]); ws[2172] = kk * CEFF_(y[41]); }
    { const double kk = ws[1327]; ws[2173] = kk * CEFF_(y[137]); ws[2174] = kk * CEFF_(y[89]); }
    { const double kk = ws[1328]; ws[2175] = kk * CEFF_(y[147]); ws[2176] = kk * CEFF_(y[89]); }
    { const double kk = ws[1329]; ws[2177] = kk * CEFF_(y[145]); ws[2178] = kk * CEFF_(y[89]); }
    { const double kk = ws[1330]; ws[2179] = kk * CEFF_(y[146]); ws[2180] = kk * CEFF_(y[89]); }
    { const double kk = ws[1331]; ws[2181] = kk * CEFF_(y[142]); ws[2182] = kk * CEFF_(y[105]); }
    { const double kk = ws[1332]; ws[2183] = kk * CEFF_(y[148]); ws[2184] = kk * CEFF_(y[105]); }
    { const double kk = ws[1341]; ws[2185] = kk * CEFF_(y[148]); ws[2186] = kk * CEFF_(y[22]); }
    { const double kk = ws[1342]; ws[2187] = kk * CEFF_(y[148]); ws[2188] = kk * CEFF_(y[45]); }
    { const double kk = ws[1343]; ws[2189] = kk * CEFF_(y[148]); ws[2190] = kk * CEFF_(y[23]); }
    { const double kk = ws[1344]; ws[2191] = kk * CEFF_(y[148]); ws[2192] = kk * CEFF_(y[46]); }
    { const double kk = ws[1345]; ws[2193] = kk * CEFF_(y[148]); ws[2194] = kk * CEFF_(y[24]); }
    { const double kk = ws[1346]; ws[2195] = kk * CEFF_(y[148]); ws[2196] = kk * CEFF_(y[86]); }
    { const double kk = ws[1347]; ws[2197] = kk * CEFF_(y[148]); ws[2198] = kk * CEFF_(y[87]); }
    { const double kk = ws[1348]; ws[2199] = kk * CEFF_(y[148]); ws[2200] = kk * CEFF_(y[88]); }
    { const double kk = ws[1349]; ws[2201] = kk * CEFF_(y[148]); ws[2202] = kk * CEFF_(y[72]); }
    { const double kk = ws[1350]; ws[2203] = kk * CEFF_(y[148]); ws[2204] = kk * CEFF_(y[47]); }
    { const double kk = ws[1351]; ws[2205] = kk * CEFF_(y[148]); ws[2206] = kk * CEFF_(y[115]); }
    { const double kk = ws[1352]; ws[2207] = kk * CEFF_(y[148]); ws[2208] = kk * CEFF_(y[116]); }
    { const double kk = ws[1353]; ws[2209] = kk * CEFF_(y[148]); ws[2210] = kk * CEFF_(y[91]); }
    { const double kk = ws[1354]; ws[2211] = kk * CEFF_(y[148]); ws[2212] = kk * CEFF_(y[99]); }
    { const double kk = ws[1355]; ws[2213] = kk * CEFF_(y[148]); ws[2214] = kk * CEFF_(y[100]); }
    { const double kk = ws[1356]; ws[2215] = kk * CEFF_(y[148]); ws[2216] = kk * CEFF_(y[73]); }
    { const double kk = ws[1357]; ws[2217] = kk * CEFF_(y[145]); ws[2218] = kk * CEFF_(y[73]); }
    { const double kk = ws[1358]; ws[2219] = kk * CEFF_(y[130]); ws[2220] = kk * CEFF_(y[73]); }
    { const double kk = ws[1361]; ws[2221] = kk * CEFF_(y[142]); ws[2222] = kk * CEFF_(y[73]); }
    { const double kk = ws[1362]; ws[2223] = kk * CEFF_(y[148]); ws[2224] = kk * CEFF_(y[74]); }
    { const double kk = ws[1363]; ws[2225] = kk * CEFF_(y[145]); ws[2226] = kk * CEFF_(y[74]); }
    { const double kk = ws[1364]; ws[2227] = kk * CEFF_(y[130]); ws[2228] = kk * CEFF_(y[74]); }
    { const double kk = ws[1366]; ws[2229] = kk * CEFF_(y[142]); ws[2230] = kk * CEFF_(y[74]); }
    { const double kk = ws[1367]; ws[2231] = kk * CEFF_(y[148]); ws[2232] = kk * CEFF_(y[75]); }
    { const double kk = ws[1368]; ws[2233] = kk * CEFF_(y[135]); ws[2234] = kk * CEFF_(y[75]); }
    { const double kk = ws[1369]; ws[2235] = kk * CEFF_(y[145]); ws[2236] = kk * CEFF_(y[75]); }
    { const double kk = ws[1370]; ws[2237] = kk * CEFF_(y[142]); ws[2238] = kk * CEFF_(y[75]); }
    { const double kk = ws[1371]; ws[2239] = kk * CEFF_(y[148]); ws[2240] = kk * CEFF_(y[76]); }
    { const double kk = ws[1372]; ws[2241] = kk * CEFF_(y[135]); ws[2242] = kk * CEFF_(y[76]); }
    { const double kk = ws[1373]; ws[2243] = kk * CEFF_(y[145]); ws[2244] = kk * CEFF_(y[76]); }
    { const double kk = ws[1375]; ws[2245] = kk * CEFF_(y[142]); ws[2246] = kk * CEFF_(y[76]); }
    { const double kk = ws[1376]; ws[2247] = kk * CEFF_(y[148]); ws[2248] = kk * CEFF_(y[93]); }
    { const double kk = ws[1377]; ws[2249] = kk * CEFF_(y[135]); ws[2250] = kk * CEFF_(y[93]); }
    { const double kk = ws[1378]; ws[2251] = kk * CEFF_(y[145]); ws[2252] = kk * CEFF_(y[93]); }
    { const double kk = ws[1380]; ws[2253] = kk * CEFF_(y[142]); ws[2254] = kk * CEFF_(y[93]); }
    { const double kk = ws[1381]; ws[2255] = kk * CEFF_(y[148]); ws[2256] = kk * CEFF_(y[48]); }
    { const double kk = ws[1382]; ws[2257] = kk * CEFF_(y[142]); ws[2258] = kk * CEFF_(y[48]); }
    { const double kk = ws[1383]; ws[2259] = kk * CEFF_(y[135]); ws[2260] = kk * CEFF_(y[94]); }
    { const double kk = ws[1384]; ws[2261] = kk * CEFF_(y[37]); ws[2262] = kk * CEFF_(y[94]); }
    { const double kk = ws[1385]; ws[2263] = kk * CEFF_(y[108]); ws[2264] = kk * CEFF_(y[94]); }
    { const double kk = ws[1386]; ws[2265] = kk * CEFF_(y[148]); ws[2266] = kk * CEFF_(y[94]); }
    { const double kk = ws[1387]; ws[2267] = kk * CEFF_(y[142]); ws[2268] = kk * CEFF_(y[94]); }
    { const double kk = ws[1388]; ws[2269] = kk * CEFF_(y[148]); ws[2270] = kk * CEFF_(y[63]); }
    { const double kk = ws[1389]; ws[2271] = kk * CEFF_(y[148]); ws[2272] = kk * CEFF_(y[63]); }
    { const double kk = ws[1390]; ws[2273] = kk * CEFF_(y[145]); ws[2274] = kk * CEFF_(y[63]); }
    { const double kk = ws[1391]; ws[2275] = kk * CEFF_(y[142]); ws[2276] = kk * CEFF_(y[63]); }
#undef CEFF_
}
}  // namespace mech_cb6r5_ae7_aq
