gbx-geometry 1
# A preshower of two thin 30 x 30 cm slabs in front of ten 50 x 50 cm
# Pb / liquid-argon layers, with a 2 cm gap between them; materials of the
# calorimeter physics file (0 vacuum, 1 Pb, 2 lAr), lengths in cm
world -40 -40 -20 40 40 60
box pre_pb 1 -15 -15 -2.0 15 15 -1.5
box pre_lar 2 -15 -15 -1.5 15 15 -0.5
box pb_0 1 -25 -25 1.5 25 25 2.0
box lar_0 2 -25 -25 2.0 25 25 3.0
box pb_1 1 -25 -25 3.0 25 25 3.5
box lar_1 2 -25 -25 3.5 25 25 4.5
box pb_2 1 -25 -25 4.5 25 25 5.0
box lar_2 2 -25 -25 5.0 25 25 6.0
box pb_3 1 -25 -25 6.0 25 25 6.5
box lar_3 2 -25 -25 6.5 25 25 7.5
box pb_4 1 -25 -25 7.5 25 25 8.0
box lar_4 2 -25 -25 8.0 25 25 9.0
box pb_5 1 -25 -25 9.0 25 25 9.5
box lar_5 2 -25 -25 9.5 25 25 10.5
box pb_6 1 -25 -25 10.5 25 25 11.0
box lar_6 2 -25 -25 11.0 25 25 12.0
box pb_7 1 -25 -25 12.0 25 25 12.5
box lar_7 2 -25 -25 12.5 25 25 13.5
box pb_8 1 -25 -25 13.5 25 25 14.0
box lar_8 2 -25 -25 14.0 25 25 15.0
box pb_9 1 -25 -25 15.0 25 25 15.5
box lar_9 2 -25 -25 15.5 25 25 16.5
