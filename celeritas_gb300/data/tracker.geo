gbx-geometry 1
# Cylindrical shells about z that are not centred on z = 0: three silicon
# layers, a PbWO4 barrel and a brass / scintillator pair; materials of the
# CMS-like physics file (0 vacuum, 1 Si, 2 PbWO4, 3 brass, 4 scintillator),
# lengths in cm
world -120 -120 -150 120 120 200
shell si_a 1 8.0 8.03 -40 60
shell si_b 1 20.0 20.03 -60 90
shell si_c 1 35.0 35.03 -80 120
shell ecal 2 50.0 72.0 -100 150
shell brass 3 80.0 85.0 -120 180
shell scint 4 85.0 85.4 -120 180
